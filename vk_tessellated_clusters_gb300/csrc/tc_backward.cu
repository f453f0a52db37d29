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
// vertex, direct atomics. Part triangles: 16 per warp; the warp walks their
// concatenated vertices, sums per (part, base vertex) in shared memory and
// adds them to the base vertex with one atomic per component; texel taps use
// global atomics.
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

// ---------------------------------------------------------------------------
// part instantiations are processed in chunks of 16 per warp: their vertices
// are contiguous, so the warp walks the flattened vertex range with all lanes
// busy (a part has ~4-80 vertices), the per-part data staged in shared memory
// ---------------------------------------------------------------------------

constexpr u32 kWarps      = 8;
constexpr u32 kChunkParts = 16;

struct PartRec
{
  f3                     bb[3];
  f3                     nh[3];  // normalised base normals
  f2                     uv[3];
  float                  nl[3];  // base normal lengths
  u32                    vi[3];
  u32                    firstVertex, cfg, inst;
  u32                    vbase;  // first generated vertex
  float                  iscale, ioffset;
  float*                 gtex;   // texel gradient of the instance's map (or null)
  tc_DisplacementTexture tx;     // width == 0: no displacement
};

struct ChunkSmem
{
  PartRec rec[kWarps][kChunkParts];
  u32     vpre[kWarps][kChunkParts + 1];
  float   acc[kWarps][kChunkParts][3][6];  // per part and base vertex: dP xyz, d(normalised normal) xyz
};

// Loads the warp's chunk [first, first + 16) of part instantiations into
// shared memory; returns the chunk's vertex count.
__device__ __forceinline__ u32 load_chunk(const StageCtx& c, float* const* gradTexels, u32 first, u32 end, PartRec* rec,
                                          u32* vpre)
{
  const u32                         lane  = threadIdx.x & 31;
  const tc_SceneBuilding*           b     = c.build;
  const tc_TemplateInstantiateInfo* ti    = reinterpret_cast<const tc_TemplateInstantiateInfo*>(b->tempInstantiations);
  const tc_TessTriangleInfo*        parts = reinterpret_cast<const tc_TessTriangleInfo*>(b->partTriangles);
  const u32                         j     = first + lane;
  u32                               nv    = 0;
  if(lane < kChunkParts && j < end)
  {
    const tc_TemplateInstantiateInfo info = ti[j];
    const tc_TessTriangleInfo pi  = parts[info.clusterIdOffset & 0x3FFFFFFFu];
    const u32                 cfg = pi.subTriangle.triangleID_config >> 16;
    const u32                 tri = pi.subTriangle.triangleID_config & 0xFFFFu;
    const tc_RenderInstance&  in  = c.instances[pi.cluster.instanceID];
    const tc_Cluster          cl  = reinterpret_cast<const tc_Cluster*>(in.clusters)[pi.cluster.clusterID];
    const uint8_t*            lt  = reinterpret_cast<const uint8_t*>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
    const tc_TessTableEntry   e   = table_entry(c.table, cfg);
    PartRec&                  r   = rec[lane];
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
      const u32 vi = cl.firstLocalVertex + lt[tri * 3 + k];
      const f3  n  = ldg3(reinterpret_cast<const float*>(in.normals), vi);
      r.vi[k]      = vi;
      r.bb[k]      = decode_bary(pi.subTriangle.vtxEncoded[k]);
      r.nl[k]      = len3(n);
      r.nh[k]      = normalize3(n);
      r.uv[k]      = ldg2(reinterpret_cast<const float*>(in.texcoords), vi);
    }
    r.firstVertex = e.firstVertex;
    r.cfg         = cfg;
    r.inst        = pi.cluster.instanceID;
    r.vbase       = (u32)((info.vertexBufferAddress - b->genVertices) / 12);
    r.iscale      = in.displacementScale;
    r.ioffset     = in.displacementOffset;
    r.tx          = {};
    r.gtex        = nullptr;
    if(c.numTextures > 0 && c.textures != nullptr && in.displacementIndex >= 0
       && (u32)in.displacementIndex < c.numTextures)
    {
      r.tx   = c.textures[in.displacementIndex];
      r.gtex = r.tx.width ? gradTexels[in.displacementIndex] : nullptr;
    }
    nv = e.numVertices;
  }
  u32 x = nv;
#pragma unroll
  for(int d = 1; d < 32; d <<= 1)
  {
    u32 y = __shfl_up_sync(0xFFFFFFFFu, x, d);
    if(lane >= (u32)d)
      x += y;
  }
  if(lane < kChunkParts)
    vpre[lane + 1] = x;
  if(lane == 0)
    vpre[0] = 0;
  __syncwarp();
  return __shfl_sync(0xFFFFFFFFu, x, kChunkParts - 1);
}

__device__ __forceinline__ u32 chunk_part_of(const u32* vpre, u32 t)
{
  u32 lo = 0, hi = kChunkParts;
#pragma unroll
  for(int s = 0; s < 4; s++)
  {
    const u32 mid = (lo + hi) >> 1;
    if(vpre[mid] <= t)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// number of leading full-cluster instantiations (they precede all parts)
__device__ __forceinline__ u32 full_count(const StageCtx& c, u32 temps)
{
  return min(c.runStarts[kMaxRuns + 1], temps);
}

__global__ void __launch_bounds__(kWarps * 32) k_instantiate_backward(StageCtx c, const float* gradVertices,
                                                                      const tc_GradTargets* targets,
                                                                      float* const* gradTexels)
{
  stage_prologue();
  __shared__ ChunkSmem sm;
  const u32         lane  = threadIdx.x & 31, warp = threadIdx.x >> 5;
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

  // part triangles (triangle_tess_template_instantiate.comp.glsl:343-371), 16 per warp
  PartRec* rec  = sm.rec[warp];
  u32*     vpre = sm.vpre[warp];
  float(*acc)[3][6] = sm.acc[warp];
  const u32 nparts  = temps - nfull;
  for(u32 chunk = gwarp; chunk * kChunkParts < nparts; chunk += nwarp)
  {
    const u32 first = nfull + chunk * kChunkParts;
    const u32 total = load_chunk(c, gradTexels, first, temps, rec, vpre);
    for(u32 t = lane; t < kChunkParts * 3 * 6; t += 32)
      (&acc[0][0][0])[t] = 0.0f;
    __syncwarp();
    for(u32 t = lane; t < total; t += 32)
    {
      const u32      pi = chunk_part_of(vpre, t);
      const PartRec& r  = rec[pi];
      const u32      v  = t - vpre[pi];
      f3             w  = decode_bary(__ldg(c.table.vertices + r.firstVertex + v));
      if(cfg_flipped(r.cfg))
      {
        const float x = w.x;
        w.x           = w.y;
        w.y           = x;
      }
      w                 = interp3(r.bb[0], r.bb[1], r.bb[2], w);
      const f3    g     = ldg3(gradVertices, (u64)r.vbase + v);
      const float wk[3] = {w.x, w.y, w.z};
#pragma unroll
      for(int k = 0; k < 3; k++)
      {
        atomicAdd(&acc[pi][k][0], wk[k] * g.x);
        atomicAdd(&acc[pi][k][1], wk[k] * g.y);
        atomicAdd(&acc[pi][k][2], wk[k] * g.z);
      }
      if(r.tx.width == 0)
        continue;
      const f3    N    = interp3(r.nh[0], r.nh[1], r.nh[2], w);
      const f2    uv   = interp2(r.uv[0], r.uv[1], r.uv[2], w);
      const float Nl   = len3(N);
      const f3    m    = normalize3(N);
      const float hraw = sample_bilinear(r.tx, uv);
      const float h    = ((hraw * r.iscale) * viewScale + r.ioffset) + viewOffset;
      const float dh   = dot3(m, g);
      // d normalize(N) / dN = (I - m m^T) / |N|
      const float kN = h / Nl;
      const f3    gN = {kN * (g.x - m.x * dh), kN * (g.y - m.y * dh), kN * (g.z - m.z * dh)};
#pragma unroll
      for(int k = 0; k < 3; k++)
      {
        atomicAdd(&acc[pi][k][3], wk[k] * gN.x);
        atomicAdd(&acc[pi][k][4], wk[k] * gN.y);
        atomicAdd(&acc[pi][k][5], wk[k] * gN.z);
      }
      if(r.gtex)
        scatter_texels(r.gtex, r.tx, bilinear_taps(r.tx, uv), dh * (r.iscale * viewScale));
    }
    __syncwarp();
    // one lane per (part, base vertex): the chunk's sums go out with 6 atomics
    const u32 nchunk = min(kChunkParts, temps - first);
    for(u32 t = lane; t < nchunk * 3; t += 32)
    {
      const u32            pi = t / 3, k = t % 3;
      const PartRec&       r  = rec[pi];
      const tc_GradTargets gt = targets[r.inst];
      const f3             dp = {acc[pi][k][0], acc[pi][k][1], acc[pi][k][2]};
      if(gt.dPositions)
        atomic_add3(reinterpret_cast<float*>(gt.dPositions), r.vi[k], dp);
      if(r.tx.width && gt.dNormals)
      {
        // d normalize(n_k) / dn_k = (I - nh nh^T) / |n_k|
        const f3    dnh = {acc[pi][k][3], acc[pi][k][4], acc[pi][k][5]};
        const f3    nh  = r.nh[k];
        const float d   = dot3(nh, dnh);
        const float rr  = 1.0f / r.nl[k];
        const f3    dn  = {rr * (dnh.x - nh.x * d), rr * (dnh.y - nh.y * d), rr * (dnh.z - nh.z * d)};
        atomic_add3(reinterpret_cast<float*>(gt.dNormals), r.vi[k], dn);
      }
    }
    __syncwarp();
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
      const u32 nv = min((u32)cl.numVertices, TC_MAX_CLUSTER_VERTICES);
      for(u32 v = lane; v < nv; v += 32)
      {
        const u32 vi = cl.firstLocalVertex + v;
        f3        p  = ldg3(reinterpret_cast<const float*>(in.positions), vi);
        if(tx.width != 0)
        {
          const float h = sample_bilinear(tx, ldg2(reinterpret_cast<const float*>(in.texcoords), vi));
          p = displace(p, ldg3(reinterpret_cast<const float*>(in.normals), vi), h, in.displacementScale, vscale,
                       in.displacementOffset, voffset);
        }
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
        f3 bp[3], bn[3];
        f2 bt[3];
#pragma unroll
        for(int k = 0; k < 3; k++)
        {
          const u32 vi = cl.firstLocalVertex + lt[tri * 3 + k];
          bp[k]        = ldg3(reinterpret_cast<const float*>(in.positions), vi);
          bn[k]        = ldg3(reinterpret_cast<const float*>(in.normals), vi);
          bt[k]        = ldg2(reinterpret_cast<const float*>(in.texcoords), vi);
        }
        write_part_affine(r, pi.subTriangle.vtxEncoded, cfg_flipped(cfg), bp, bn, bt, e.firstVertex, tx,
                          in.displacementScale * vscale, in.displacementOffset + voffset);
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
