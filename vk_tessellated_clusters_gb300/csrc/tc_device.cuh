// tc_device.cuh — device-side building blocks shared by all kernels.
//
// Arithmetic contract: the library is compiled with -fmad=false and IEEE
// division/square root, and every expression below is written in the
// evaluation order of the reference GLSL (left to right), so results are
// bit-identical to the oracle's (g++ -ffp-contract=off).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include "tc_tessellation.h"

namespace tc {

typedef unsigned long long u64;
typedef uint32_t           u32;

// ---------------------------------------------------------------------------
// vectors
// ---------------------------------------------------------------------------

struct f3
{
  float x, y, z;
};
struct f2
{
  float x, y;
};

__device__ __forceinline__ f3 ldg3(const float* base, u64 index)
{
  const float* p = base + 3 * index;
  return {__ldg(p), __ldg(p + 1), __ldg(p + 2)};
}
__device__ __forceinline__ f2 ldg2(const float* base, u64 index)
{
  const float2 v = __ldg(reinterpret_cast<const float2*>(base) + index);
  return {v.x, v.y};
}

__device__ __forceinline__ f3    sub3(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float len3(f3 a) { return __fsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ float dist3(f3 a, f3 b) { return len3(sub3(a, b)); }
// GLSL normalize(): v * (1 / length(v)) (one IEEE division, three multiplies)
__device__ __forceinline__ f3 normalize3(f3 a)
{
  float r = __fdiv_rn(1.0f, len3(a));
  return {a.x * r, a.y * r, a.z * r};
}

// (M * vec4(p, 1)).xyz, column-major M
__device__ __forceinline__ f3 xform_point(const float* m, f3 p)
{
  f3 r;
  r.x = ((m[0] * p.x + m[4] * p.y) + m[8] * p.z) + m[12];
  r.y = ((m[1] * p.x + m[5] * p.y) + m[9] * p.z) + m[13];
  r.z = ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14];
  return r;
}

// tessellation.glsl:191-201 tess_interpolate (precise)
__device__ __forceinline__ f3 interp3(f3 b0, f3 b1, f3 b2, f3 w)
{
  f3 r;
  r.x = (b0.x * w.x + b1.x * w.y) + b2.x * w.z;
  r.y = (b0.y * w.x + b1.y * w.y) + b2.y * w.z;
  r.z = (b0.z * w.x + b1.z * w.y) + b2.z * w.z;
  return r;
}
__device__ __forceinline__ f2 interp2(f2 b0, f2 b1, f2 b2, f3 w)
{
  f2 r;
  r.x = (b0.x * w.x + b1.x * w.y) + b2.x * w.z;
  r.y = (b0.y * w.x + b1.y * w.y) + b2.y * w.z;
  return r;
}

// ---------------------------------------------------------------------------
// tessellation.glsl
// ---------------------------------------------------------------------------

// tessellation.glsl:48-59
__device__ __forceinline__ u32 encode_bary(f3 w)
{
  u32 ix = __float2uint_rz(w.x * 32768.0f + 0.5f);
  u32 iy = __float2uint_rz(w.y * 32768.0f + 0.5f);
  u32 iz = __float2uint_rz(w.z * 32768.0f + 0.5f);
  if(ix > max(iy, iz))
    ix = 32768u - iy - iz;
  else if(iy > iz)
    iy = 32768u - ix - iz;
  else
    iz = 32768u - ix - iy;
  return iy | (iz << 16);
}

// tessellation.glsl:66-76
__device__ __forceinline__ f3 decode_bary(u32 vtx)
{
  f3 w;
  w.y = __uint2float_rn(vtx & 0xFFFFu) * (1.0f / 32768.0f);
  w.z = __uint2float_rn(vtx >> 16) * (1.0f / 32768.0f);
  w.x = (1.0f - w.y) - w.z;
  return w;
}

struct FactorParams
{
  f3    viewPos;
  float nearPlane;
  float viewportH;
  float tessRate;
};

__device__ __forceinline__ u32 round_clamp_factor(float e, float spl, const FactorParams& fp)
{
  float f = rintf(((e * spl) * fp.viewportH) * fp.tessRate);
  f       = fminf(fmaxf(f, 1.0f), 32768.0f);
  return __float2uint_rz(f);
}

// tessellation.glsl:78-99
__device__ __forceinline__ uint3 tess_factors(f3 a, f3 b, f3 c, const FactorParams& fp)
{
  float da = dist3(a, fp.viewPos);
  float db = dist3(b, fp.viewPos);
  float dc = dist3(c, fp.viewPos);
  float sx = __fdiv_rn(1.0f, fmaxf(fp.nearPlane, fminf(da, db)));
  float sy = __fdiv_rn(1.0f, fmaxf(fp.nearPlane, fminf(db, dc)));
  float sz = __fdiv_rn(1.0f, fmaxf(fp.nearPlane, fminf(dc, da)));
  uint3 f;
  f.x = round_clamp_factor(dist3(a, b), sx, fp);
  f.y = round_clamp_factor(dist3(b, c), sy, fp);
  f.z = round_clamp_factor(dist3(c, a), sz, fp);
  return f;
}

// tess_factors with the per-vertex work hoisted: d_k = |p_k - viewPos| and
// r_k = 1 / d_k (IEEE division) computed once per vertex, rNear = 1 / nearPlane.
// Division is monotonic, so 1 / max(near, min(d_a, d_b)) is exactly the
// reciprocal of whichever of near, d_a, d_b the max/min selects: the same bits
// as tess_factors.
__device__ __forceinline__ float rcp_of_clamped_min(float da, float db, float ra, float rb, float nearPlane, float rNear)
{
  const float m  = fminf(da, db);
  const float rm = da <= db ? ra : rb;
  return nearPlane > m ? rNear : rm;
}

// The factor of edge a-b, round_clamp_factor(|a - b|, spl, fp), without the
// square root where the answer is certainly 1. That factor is 1 exactly when
// x = ((|a - b| * spl) * viewportH) * tessRate is below 1.5 (rint then gives
// at most 1). t = (|a - b|^2 * spl^2) * (viewportH * tessRate)^2 in single
// precision carries five roundings (relative error below 3.0e-7) and x four
// (below 2.4e-7), so t < 2.25 * (1 - 1e-5) puts x below 1.5 * (1 - 4.6e-6):
// the factor is 1, the same result as the full evaluation. Every other edge
// (and NaN or infinite t) takes the full evaluation, on the same |a - b|^2.
constexpr float kFactorOneBound = 2.2499775f;  // 2.25 * (1 - 1e-5)

__device__ __forceinline__ u32 edge_factor(f3 a, f3 b, float spl, float k2, const FactorParams& fp)
{
  const f3    d  = sub3(a, b);
  const float s2 = dot3(d, d);
  if((s2 * (spl * spl)) * k2 < kFactorOneBound)
    return 1u;
  return round_clamp_factor(__fsqrt_rn(s2), spl, fp);
}

// edge_factor's test from squared quantities alone: da2, db2 are the squared
// distances of a and b to the view position (tess_factors_hoisted takes their
// square roots as da, db), near2 = nearPlane^2, k2 = (viewportH * tessRate)^2.
// With u = 2^-24 and Q = max(nearPlane, min(sqrt(da2), sqrt(db2))): the left
// side is at least |a - b|^2 * (viewportH * tessRate)^2 * (1 - u)^4, the
// right side at most 2.25 * (1 - 1e-5) * Q^2 * (1 + u)^2, and the factor's
// product x at most |a - b| / Q * viewportH * tessRate * (1 + u)^6 (the
// roots, the reciprocal and three products), so a true test puts x below
// 1.5 * (1 - 5e-6 + 9u) < 1.5: the factor is 1. NaN and infinite values fail
// the test (or give x = 0 and the factor 1 as well).
__device__ __forceinline__ bool edge_factor_one_sq(f3 a, f3 b, float da2, float db2, float k2, float near2)
{
  const f3    d  = sub3(a, b);
  const float s2 = dot3(d, d);
  return s2 * k2 < kFactorOneBound * fmaxf(near2, fminf(da2, db2));
}

__device__ __forceinline__ uint3 tess_factors_hoisted(f3 a, f3 b, f3 c, float da, float db, float dc, float ra, float rb,
                                                      float rc, float rNear, const FactorParams& fp)
{
  const float sx = rcp_of_clamped_min(da, db, ra, rb, fp.nearPlane, rNear);
  const float sy = rcp_of_clamped_min(db, dc, rb, rc, fp.nearPlane, rNear);
  const float sz = rcp_of_clamped_min(dc, da, rc, ra, fp.nearPlane, rNear);
  const float k  = fp.viewportH * fp.tessRate;
  const float k2 = k * k;
  uint3       f;
  f.x = edge_factor(a, b, sx, k2, fp);
  f.y = edge_factor(b, c, sy, k2, fp);
  f.z = edge_factor(c, a, sz, k2, fp);
  return f;
}

// tessellation.glsl:101-104
__device__ __forceinline__ u32 split_factor1(u32 f, u32 sf) { return min((f + TC_TESSTABLE_SIZE - 1) / TC_TESSTABLE_SIZE, sf); }

// tessellation.glsl:119-144: rotate the largest factor first (permuting the
// three encoded sub-triangle vertices with it), flip bit when z > y
__device__ __forceinline__ u32 get_config(uint3 f, u32& v0, u32& v1, u32& v2)
{
  u32 m = max(max(f.x, f.y), f.z);
  if(m == f.y)
  {
    f       = make_uint3(f.y, f.z, f.x);
    u32 t0 = v0;
    v0 = v1, v1 = v2, v2 = t0;
  }
  else if(m == f.z)
  {
    f       = make_uint3(f.z, f.x, f.y);
    u32 t2 = v2;
    v2 = v1, v1 = v0, v0 = t2;
  }
  const u32 L   = TC_TESSTABLE_LOOKUP_SIZE;
  u32       idx = f.x + f.y * L + f.z * L * L - (1 + L + L * L);
  if(f.z > f.y)
    idx |= 1u << 15;
  return idx;
}

__device__ __forceinline__ u32  cfg_index(u32 cfg) { return cfg & 0x7FFFu; }
__device__ __forceinline__ bool cfg_flipped(u32 cfg) { return (cfg & 0x8000u) != 0; }

struct Table
{
  const tc_TessTableEntry* entries;
  const u32*               vertices;
  const u32*               triangles;
  const u64*               templateAddresses;
  const u32*               templateSizes;
};

__device__ __forceinline__ tc_TessTableEntry table_entry(const Table& t, u32 cfg)
{
  const uint2 raw = __ldg(reinterpret_cast<const uint2*>(t.entries) + cfg_index(cfg));
  tc_TessTableEntry e;
  e.firstTriangle = raw.x & 0xFFFF;
  e.firstVertex   = raw.x >> 16;
  e.numTriangles  = raw.y & 0xFFFF;
  e.numVertices   = raw.y >> 16;
  return e;
}

// tessellation.glsl:165-176 (flip -> .xzy)
__device__ __forceinline__ uint3 cfg_triangle(const Table& t, const tc_TessTableEntry& e, u32 cfg, u32 tri)
{
  u32   p = __ldg(t.triangles + e.firstTriangle + tri);
  uint3 r = make_uint3(p & 0xFF, (p >> 8) & 0xFF, (p >> 16) & 0xFF);
  if(cfg_flipped(cfg))
  {
    u32 s = r.y;
    r.y   = r.z;
    r.z   = s;
  }
  return r;
}

// tessellation.glsl:178-189 (flip -> .yxz)
__device__ __forceinline__ f3 cfg_vertex(const Table& t, const tc_TessTableEntry& e, u32 cfg, u32 vert)
{
  f3 w = decode_bary(__ldg(t.vertices + e.firstVertex + vert));
  if(cfg_flipped(cfg))
  {
    float s = w.x;
    w.x     = w.y;
    w.y     = s;
  }
  return w;
}

// ---------------------------------------------------------------------------
// displacement: bilinear, mip 0, REPEAT, texel centres at (i + 0.5) / size.
// Texels are fetched with read-only (texture-path) loads; weights are fp32 and
// computed here, so the result does not depend on the sampler's fixed-point
// filter weights.
// ---------------------------------------------------------------------------

// i mod n in [0, n); taps are almost always within one period of the range
__device__ __forceinline__ int wrapi(int i, int n)
{
  if((unsigned)i < (unsigned)n)
    return i;
  if(i < 0 && i >= -n)
    return i + n;
  if(i >= n && i - n < n)
    return i - n;
  int r = i % n;
  return r < 0 ? r + n : r;
}

__device__ __forceinline__ float fetch_texel(const tc_DisplacementTexture& tx, int x, int y)
{
  const u64 i = (u64)y * tx.width + (u64)x;
  switch(tx.format)
  {
    case TC_TEXEL_F16:
      return __half2float(__ushort_as_half(__ldg(reinterpret_cast<const unsigned short*>(tx.texels) + i)));
    case TC_TEXEL_UNORM16:
      return __fdiv_rn(__uint2float_rn(__ldg(reinterpret_cast<const unsigned short*>(tx.texels) + i)), 65535.0f);
    default:
      return __ldg(reinterpret_cast<const float*>(tx.texels) + i);
  }
}

struct Taps
{
  int   x0, x1, y0, y1;
  float fx, fy;
};

__device__ __forceinline__ Taps bilinear_taps(const tc_DisplacementTexture& tx, f2 uv)
{
  float x  = uv.x * __uint2float_rn(tx.width) - 0.5f;
  float y  = uv.y * __uint2float_rn(tx.height) - 0.5f;
  float xf = floorf(x);
  float yf = floorf(y);
  Taps  t;
  t.fx   = x - xf;
  t.fy   = y - yf;
  int ix = __float2int_rz(xf), iy = __float2int_rz(yf);
  t.x0   = wrapi(ix, (int)tx.width);
  t.x1   = wrapi(ix + 1, (int)tx.width);
  t.y0   = wrapi(iy, (int)tx.height);
  t.y1   = wrapi(iy + 1, (int)tx.height);
  return t;
}

__device__ __forceinline__ float sample_bilinear(const tc_DisplacementTexture& tx, f2 uv)
{
  if(tx.width == 0 || tx.height == 0)
    return 0.0f;
  Taps      b  = bilinear_taps(tx, uv);
  const u64 r0 = (u64)b.y0 * tx.width, r1 = (u64)b.y1 * tx.width;
  float     t00, t10, t01, t11;
  if(tx.format == TC_TEXEL_F16)
  {
    const unsigned short* t = reinterpret_cast<const unsigned short*>(tx.texels);
    t00 = __half2float(__ushort_as_half(__ldg(t + r0 + b.x0)));
    t10 = __half2float(__ushort_as_half(__ldg(t + r0 + b.x1)));
    t01 = __half2float(__ushort_as_half(__ldg(t + r1 + b.x0)));
    t11 = __half2float(__ushort_as_half(__ldg(t + r1 + b.x1)));
  }
  else if(tx.format == TC_TEXEL_F32)
  {
    const float* t = reinterpret_cast<const float*>(tx.texels);
    t00 = __ldg(t + r0 + b.x0);
    t10 = __ldg(t + r0 + b.x1);
    t01 = __ldg(t + r1 + b.x0);
    t11 = __ldg(t + r1 + b.x1);
  }
  else
  {
    t00 = fetch_texel(tx, b.x0, b.y0);
    t10 = fetch_texel(tx, b.x1, b.y0);
    t01 = fetch_texel(tx, b.x0, b.y1);
    t11 = fetch_texel(tx, b.x1, b.y1);
  }
  float gx = 1.0f - b.fx;
  float top = gx * t00 + b.fx * t10;
  float bot = gx * t01 + b.fx * t11;
  return (1.0f - b.fy) * top + b.fy * bot;
}

// height = (h * instScale * viewScale) + instOffset + viewOffset; pos += normalize(n) * height
// (cluster_classify.comp.glsl:471-478, triangle_tess_template_instantiate.comp.glsl:356-365)
__device__ __forceinline__ f3 displace(f3 pos, f3 normal, float h, float instScale, float viewScale, float instOffset,
                                       float viewOffset)
{
  h    = ((h * instScale) * viewScale + instOffset) + viewOffset;
  f3 n = normalize3(normal);
  return {pos.x + n.x * h, pos.y + n.y * h, pos.z + n.z * h};
}

// ---------------------------------------------------------------------------
// memory-model helpers
// ---------------------------------------------------------------------------

// Look-back state words carry their value and flag in one 64-bit word and
// nothing else is published through them, so relaxed (single-copy atomic)
// accesses at GPU scope suffice: no fences on the polling path.
__device__ __forceinline__ void st_relaxed_u64(u64* p, u64 v)
{
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ u64 ld_relaxed_u64(const u64* p)
{
  u64 v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ u32 ld_acquire_u32(const u32* p)
{
  u32 v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// ---------------------------------------------------------------------------
// Programmatic dependent launch. Every stage kernel is launched with
// programmatic stream serialisation (launch_pdl in tc_stage.cuh): it may be
// scheduled while its predecessor in the stream is still running, so its
// launch latency and block start-up overlap the predecessor's tail. Each
// kernel opens with stage_prologue(): it lets its own successor launch early
// (the trigger fires once every block of this grid has started, so a waiting
// successor never holds resources a not-yet-started block needs), then waits
// for the full completion and memory visibility of its predecessor before it
// touches global memory. Completion is transitive: a kernel completes only
// after passing its own wait.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void stage_prologue()
{
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ---------------------------------------------------------------------------
// Decoupled look-back (single-pass chained scan) over tiles. Gives every tile
// the exclusive prefix of per-tile aggregates in tile order, so appends are
// ordered exactly like a serial loop. Each state word holds a 62-bit value and
// a 2-bit flag (1 = tile aggregate, 2 = inclusive prefix). Tiles are handed out
// through a ticket counter so a tile's predecessors are always owned by running
// blocks. Waits are bounded: after `spinLimit` polls (the schedule's
// lookbackSpinLimit, by default kSpinLimit) the tile records
// TC_DEVERR_LOOKBACK_TIMEOUT, uses what it accumulated and moves on.
// ---------------------------------------------------------------------------

constexpr u64 kLbValueMask = (1ull << 62) - 1;
constexpr u64 kLbAggregate = 1ull << 62;
constexpr u64 kLbPrefix    = 2ull << 62;
constexpr u32 kSpinLimit   = 1u << 22;

__device__ __forceinline__ u64 warp_sum_u64(u64 v)
{
#pragma unroll
  for(int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// Warp-cooperative look-back: all 32 lanes of one warp call it for one counter
// and all receive the tile's exclusive prefix. Each step reads a window of the
// kLbWindow = 128 nearest predecessors at once (lane i reads tiles
// tile - 1 - i - 32 k, k = 0..3: four independent loads per lane, one round
// trip), waits until all of them have published, and either stops at the
// nearest inclusive prefix or adds the aggregates and moves the window back.
// The prefix frontier therefore advances 128 tiles per memory round trip.
// `state` is this counter's tile-state array; `base` (the counter value before
// this launch) is only used by tile 0.
constexpr int kLbSlots      = 4;
constexpr int kLbWindow     = 32 * kLbSlots;
constexpr u32 kLbEagerPolls = 64;

__device__ __forceinline__ u64 warp_lookback_exclusive(u64* state, u32 tile, u64 aggregate, u64 base, u32* errorWord,
                                                        u32 spinLimit)
{
  const u32 lane = threadIdx.x & 31;
  if(tile == 0)
  {
    if(lane == 0)
      st_relaxed_u64(state, kLbPrefix | ((base + aggregate) & kLbValueMask));
    return base;
  }
  if(lane == 0)
    st_relaxed_u64(state + tile, kLbAggregate | (aggregate & kLbValueMask));
  u64 excl  = 0;
  int start = (int)tile - 1;
  u32 spins = 0;
  for(;;)
  {
    u64 s[kLbSlots];
#pragma unroll
    for(int k = 0; k < kLbSlots; k++)
    {
      const int t = start - (int)lane - 32 * k;
      // window slots before tile 0 count as an empty inclusive prefix
      s[k] = t >= 0 ? ld_relaxed_u64(state + t) : kLbPrefix;
    }
    for(;;)
    {
      bool pending = false;
#pragma unroll
      for(int k = 0; k < kLbSlots; k++)
        pending |= (s[k] & ~kLbValueMask) == 0;
      if(!__any_sync(0xFFFFFFFFu, pending))
        break;
      if(++spins > spinLimit)
      {
        if(lane == 0)
          atomicOr(errorWord, TC_DEVERR_LOOKBACK_TIMEOUT);
#pragma unroll
        for(int k = 0; k < kLbSlots; k++)
          if((s[k] & ~kLbValueMask) == 0)
            s[k] = kLbPrefix;  // give up on this window
        break;
      }
      // predecessors usually publish within a few hundred nanoseconds: poll
      // back to back at first, then back off
      if(spins > kLbEagerPolls)
        __nanosleep(spins > 4 * kLbEagerPolls ? 256 : 32);
#pragma unroll
      for(int k = 0; k < kLbSlots; k++)
        if((s[k] & ~kLbValueMask) == 0)
          s[k] = ld_relaxed_u64(state + (start - (int)lane - 32 * k));
    }
    // nearest slot (smallest window index 32 k + lane) holding an inclusive prefix
    int first = kLbWindow;
#pragma unroll
    for(int k = kLbSlots - 1; k >= 0; k--)
    {
      const u32 pmask = __ballot_sync(0xFFFFFFFFu, (s[k] & ~kLbValueMask) == kLbPrefix);
      if(pmask)
        first = 32 * k + __ffs(pmask) - 1;
    }
    u64 v = 0;
#pragma unroll
    for(int k = 0; k < kLbSlots; k++)
      if(32 * k + (int)lane <= first)
        v += s[k] & kLbValueMask;
    excl += warp_sum_u64(v);
    if(first < kLbWindow)
      break;
    start -= kLbWindow;
  }
  if(lane == 0)
    st_relaxed_u64(state + tile, kLbPrefix | ((excl + aggregate) & kLbValueMask));
  return excl;
}

// binary search: first index in [lo, hi) whose instance id (read by `get`) is >= key
template <class Get>
__device__ __forceinline__ u32 lower_bound_instance(u32 lo, u32 hi, u32 key, Get get)
{
  while(lo < hi)
  {
    u32 mid = lo + ((hi - lo) >> 1);
    if(get(mid) < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

}  // namespace tc
