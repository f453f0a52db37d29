// tc_vertex.cuh — displaced vertex of a part triangle in per-part affine form.
//
// The reference (triangle_tess_template_instantiate.comp.glsl:343-371) maps
// each table vertex w of the config through the part's sub-triangle corners
// bb_k into base-triangle barycentrics, interpolates position, normalised
// normal and uv with them, samples the displacement map and displaces along
// the renormalised normal. Both interpolations are linear, so for a table
// vertex w = (1 - a - b, a, b) every attribute is
//
//     A(w) = A_0 + a (A_1 - A_0) + b (A_2 - A_0),   A_k = sum_j C_k[j] attr_j
//
// with C_k the sub-triangle corners (a flipped config swaps C_0 and C_1, the
// same as swapping w.x and w.y). A_k are evaluated once per part; a vertex then
// costs three fused multiply-adds per component. The result equals the
// reference's two-level evaluation up to rounding (a few ulps of the
// coordinates), inside the |dp| <= 1e-5 x bounding-box-diagonal tolerance the
// positions are held to; integer outputs are unaffected.
//
// Bilinear displacement: mip 0, REPEAT, texel centres at (i + 0.5) / size,
// fp32 weights, texels through read-only loads (one path for fp32, fp16 and
// unorm16 maps).
#pragma once

#include "tc_device.cuh"

namespace tc {

// Nine 16-byte words read with vector loads from shared memory; the 144-byte
// stride puts consecutive records of an array in different bank groups.
struct __align__(16) PartAffine
{
  float4 q[9];
  // q[0] = P0.xyz, E1.x       P0 = position at corner 0, E1 = P1 - P0, E2 = P2 - P0
  // q[1] = E1.yz, E2.xy
  // q[2] = E2.z, N0.xyz       N = interpolated normalised base normals
  // q[3] = F1.xyz, F2.x       F1 = N1 - N0, F2 = N2 - N0
  // q[4] = F2.yz, T0.xy       T = uv
  // q[5] = G1.xy, G2.xy       G1 = T1 - T0, G2 = T2 - T0
  // q[6] = scale, offset, firstVertex (bits), kind (bits; see affine_kind)
  // q[7] = texels lo, texels hi, width, height (bits; width 0 = no displacement)
  // q[8] = width, height (as floats), width - 1, height - 1 (bits; the wrap
  //        masks of power-of-two sizes)
};

// Record kinds (q[6].w): what the vertex needs beyond the interpolated position.
enum : u32
{
  kAffineFlat     = 0,  // no displacement map
  kAffineZeroMap  = 1,  // map of height 0: displaced by the offsets only
  kAffineTextured = 2,  // 2 + 2 * format + (1 if both sizes are powers of two)
};

__host__ __device__ constexpr u32 affine_kind(u32 format, bool pow2) { return kAffineTextured + 2 * format + (pow2 ? 1 : 0); }

// A displacement map as the vertex code reads it: q7 = texels lo, texels hi,
// width, height (bits); q8 = width, height (floats), width - 1, height - 1
// (bits; the wrap masks of power-of-two sizes); kind = affine_kind(format, pow2),
// kAffineFlat without a map, kAffineZeroMap for a map of height 0.
struct MapDesc
{
  float4 q7, q8;
  u32    kind;
};

__device__ __forceinline__ MapDesc make_map_desc(const tc_DisplacementTexture& tx)
{
  MapDesc   m;
  const u32 w = tx.width, h = tx.height;
  m.q7 = w ? make_float4(__uint_as_float((u32)tx.texels), __uint_as_float((u32)(tx.texels >> 32)), __uint_as_float(w),
                         __uint_as_float(h))
           : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  m.q8 = make_float4(__uint2float_rn(w), __uint2float_rn(h), __uint_as_float(w - 1), __uint_as_float(h - 1));
  const bool pow2 = w != 0 && h != 0 && (w & (w - 1)) == 0 && (h & (h - 1)) == 0;
  // formats other than fp16 / unorm16 read as fp32, as in every other sampling path
  const u32 fmt = tx.format == TC_TEXEL_F16 || tx.format == TC_TEXEL_UNORM16 ? tx.format : TC_TEXEL_F32;
  m.kind        = w == 0 ? kAffineFlat : (h == 0 ? kAffineZeroMap : affine_kind(fmt, pow2));
  return m;
}

__device__ __forceinline__ f3 fma3(float s, f3 a, f3 b)
{
  return {__fmaf_rn(s, a.x, b.x), __fmaf_rn(s, a.y, b.y), __fmaf_rn(s, a.z, b.z)};
}

// sum_j c[j] v_j
__device__ __forceinline__ f3 bary3(f3 c, f3 v0, f3 v1, f3 v2) { return fma3(c.z, v2, fma3(c.y, v1, {c.x * v0.x, c.x * v0.y, c.x * v0.z})); }
__device__ __forceinline__ f2 bary2(f3 c, f2 v0, f2 v1, f2 v2)
{
  return {__fmaf_rn(c.z, v2.x, __fmaf_rn(c.y, v1.x, c.x * v0.x)), __fmaf_rn(c.z, v2.y, __fmaf_rn(c.y, v1.y, c.x * v0.y))};
}

// normalize(v) as v * rsqrt(dot(v, v)) (hardware reciprocal square root)
__device__ __forceinline__ f3 normalize_fast(f3 v)
{
  const float k = rsqrtf(__fmaf_rn(v.z, v.z, __fmaf_rn(v.y, v.y, v.x * v.x)));
  return {v.x * k, v.y * k, v.z * k};
}

// Per-part set-up, written straight into `r` (normally shared memory) word by
// word. `corner` are the sub-triangle's encoded corners
// (TessTriangleInfo.vtxEncoded), p / n / uv the base triangle's positions,
// normals (normalised here, triangle_tess_template_instantiate.comp.glsl:329)
// and uvs; `scale` / `offset` the combined displacement scale (instance x
// view) and offset (instance + view).
__device__ __forceinline__ void write_part_affine(PartAffine& r, const u32 corner[3], bool flipped, const f3 p[3],
                                                  const f3 n[3], const f2 uv[3], u32 firstVertex,
                                                  const tc_DisplacementTexture& tx, float scale, float offset)
{
  f3 c0 = decode_bary(corner[0]), c1 = decode_bary(corner[1]), c2 = decode_bary(corner[2]);
  if(flipped)
  {
    const f3 t = c0;
    c0         = c1;
    c1         = t;
  }
  const u32     w = tx.width;
  const MapDesc m = make_map_desc(tx);
  r.q[6]          = make_float4(scale, offset, __uint_as_float(firstVertex), __uint_as_float(m.kind));
  r.q[7]          = m.q7;
  r.q[8]          = m.q8;
  {
    const f3 P0 = bary3(c0, p[0], p[1], p[2]);
    const f3 E1 = sub3(bary3(c1, p[0], p[1], p[2]), P0);
    r.q[0]      = make_float4(P0.x, P0.y, P0.z, E1.x);
    const f3 E2 = sub3(bary3(c2, p[0], p[1], p[2]), P0);
    r.q[1]      = make_float4(E1.y, E1.z, E2.x, E2.y);
    r.q[2].x    = E2.z;
  }
  if(w == 0)
    return;
  const f3 nh[3] = {normalize_fast(n[0]), normalize_fast(n[1]), normalize_fast(n[2])};
  const f3 N0    = bary3(c0, nh[0], nh[1], nh[2]);
  r.q[2]      = make_float4(r.q[2].x, N0.x, N0.y, N0.z);
  const f3 F1 = sub3(bary3(c1, nh[0], nh[1], nh[2]), N0);
  const f3 F2 = sub3(bary3(c2, nh[0], nh[1], nh[2]), N0);
  r.q[3]      = make_float4(F1.x, F1.y, F1.z, F2.x);
  const f2 T0 = bary2(c0, uv[0], uv[1], uv[2]), T1 = bary2(c1, uv[0], uv[1], uv[2]), T2 = bary2(c2, uv[0], uv[1], uv[2]);
  r.q[4]      = make_float4(F2.y, F2.z, T0.x, T0.y);
  r.q[5]      = make_float4(T1.x - T0.x, T1.y - T0.y, T2.x - T0.x, T2.y - T0.y);
}

// Encoded unit barycentrics: (1,0,0) -> 0, (0,1,0) -> 1, (0,0,1) -> 2, anything else -> 3.
__device__ __forceinline__ u32 unit_corner(u32 e)
{
  return e == 0u ? 0u : (e == TC_TESSTABLE_COORD_MAX ? 1u : (e == (TC_TESSTABLE_COORD_MAX << 16) ? 2u : 3u));
}

// Every part classify writes is a whole base triangle: its three corners are
// the base triangle's own corners, in the order get_config rotated them. Then
// each corner's composed attribute (the barycentric composition of
// write_part_affine) is exactly one base vertex's attribute, so the affine
// form is the base attributes themselves, taken in corner order. Returns true
// for such a part, with order[k] = the base vertex of corner k (a flipped
// config swaps corners 0 and 1); otherwise order = {0, 1, 2}.
__device__ __forceinline__ bool whole_triangle_order(const u32 corner[3], bool flipped, u32 order[3])
{
  u32        m0 = unit_corner(corner[0]), m1 = unit_corner(corner[1]), m2 = unit_corner(corner[2]);
  const bool whole = max(m0, max(m1, m2)) < 3u && m0 != m1 && m1 != m2 && m0 != m2;
  if(!whole)
    m0 = 0, m1 = 1, m2 = 2;
  else if(flipped)
  {
    const u32 t = m0;
    m0          = m1;
    m1          = t;
  }
  order[0] = m0, order[1] = m1, order[2] = m2;
  return whole;
}

// write_part_affine for a whole-triangle part whose base attributes p / n /
// uv are given in corner order: no compositions (the same values up to the
// sign of exact zeros).
__device__ __forceinline__ void write_part_affine_whole(PartAffine& r, const f3 p[3], const f3 n[3], const f2 uv[3],
                                                        u32 firstVertex, const tc_DisplacementTexture& tx, float scale,
                                                        float offset)
{
  const u32     w = tx.width;
  const MapDesc m = make_map_desc(tx);
  r.q[6]          = make_float4(scale, offset, __uint_as_float(firstVertex), __uint_as_float(m.kind));
  r.q[7]          = m.q7;
  r.q[8]          = m.q8;
  const f3 E1     = sub3(p[1], p[0]), E2 = sub3(p[2], p[0]);
  r.q[0]          = make_float4(p[0].x, p[0].y, p[0].z, E1.x);
  r.q[1]          = make_float4(E1.y, E1.z, E2.x, E2.y);
  r.q[2].x        = E2.z;
  if(w == 0)
    return;
  const f3 N0 = normalize_fast(n[0]), N1 = normalize_fast(n[1]), N2 = normalize_fast(n[2]);
  const f3 F1 = sub3(N1, N0), F2 = sub3(N2, N0);
  r.q[2]      = make_float4(E2.z, N0.x, N0.y, N0.z);
  r.q[3]      = make_float4(F1.x, F1.y, F1.z, F2.x);
  r.q[4]      = make_float4(F2.y, F2.z, uv[0].x, uv[0].y);
  r.q[5]      = make_float4(uv[1].x - uv[0].x, uv[1].y - uv[0].y, uv[2].x - uv[0].x, uv[2].y - uv[0].y);
}

// The affine form of part triangle `pt` (cluster / instance resolved by the
// caller): base attributes loaded in corner order for a whole-triangle part,
// else in base order and composed with the corners.
__device__ __forceinline__ void part_affine(PartAffine& r, const u32 corner[3], bool flipped, const float* pos,
                                            const float* nrm, const float* uvs, u32 firstLocalVertex,
                                            const uint8_t* triIndices, u32 firstVertex, const tc_DisplacementTexture& tx,
                                            float scale, float offset)
{
  u32        order[3];
  const bool whole = whole_triangle_order(corner, flipped, order);
  f3         bp[3], bn[3];
  f2         bt[3];
#pragma unroll
  for(int v = 0; v < 3; v++)
  {
    const u32 vi = firstLocalVertex + triIndices[order[v]];
    bp[v]        = ldg3(pos, vi);
    bn[v]        = ldg3(nrm, vi);  // normalised in write_part_affine* (triangle_tess_template_instantiate.comp.glsl:329)
    bt[v]        = ldg2(uvs, vi);
  }
  if(whole)
    write_part_affine_whole(r, bp, bn, bt, firstVertex, tx, scale, offset);
  else
    write_part_affine(r, corner, flipped, bp, bn, bt, firstVertex, tx, scale, offset);
}

template <u32 Format>
__device__ __forceinline__ float texel_at(u64 texels, u64 i)
{
  if(Format == TC_TEXEL_F16)
    return __half2float(__ushort_as_half(__ldg(reinterpret_cast<const unsigned short*>(texels) + i)));
  if(Format == TC_TEXEL_F32)
    return __ldg(reinterpret_cast<const float*>(texels) + i);
  return __uint2float_rn(__ldg(reinterpret_cast<const unsigned short*>(texels) + i)) * (1.0f / 65535.0f);
}

// bilinear sample at (u, v) of the map described by q7 and q8
template <u32 Format, bool Pow2>
__device__ __forceinline__ float affine_sample(float4 q7, float4 q8, float u, float v)
{
  const u32   w = __float_as_uint(q7.z), h = __float_as_uint(q7.w);
  const float x = __fmaf_rn(u, q8.x, -0.5f), y = __fmaf_rn(v, q8.y, -0.5f);
  const float xf = floorf(x), yf = floorf(y);
  const float fx = x - xf, fy = y - yf;
  const int   ix = __float2int_rz(xf), iy = __float2int_rz(yf);
  int         x0, x1, y0, y1;
  if(Pow2)
  {
    const int mx = (int)__float_as_uint(q8.z), my = (int)__float_as_uint(q8.w);
    x0 = ix & mx, x1 = (ix + 1) & mx, y0 = iy & my, y1 = (iy + 1) & my;
  }
  else
  {
    x0 = wrapi(ix, (int)w), x1 = wrapi(ix + 1, (int)w), y0 = wrapi(iy, (int)h), y1 = wrapi(iy + 1, (int)h);
  }
  const u64   texels = (u64)__float_as_uint(q7.x) | ((u64)__float_as_uint(q7.y) << 32);
  const u32   r0 = (u32)y0 * w, r1 = (u32)y1 * w;  // maps hold fewer than 2^32 texels
  const float t00 = texel_at<Format>(texels, r0 + (u32)x0), t10 = texel_at<Format>(texels, r0 + (u32)x1);
  const float t01 = texel_at<Format>(texels, r1 + (u32)x0), t11 = texel_at<Format>(texels, r1 + (u32)x1);
  const float top = __fmaf_rn(fx, t10 - t00, t00), bot = __fmaf_rn(fx, t11 - t01, t01);
  return __fmaf_rn(fy, bot - top, top);
}

__device__ __forceinline__ u32 affine_kind_of(const PartAffine& r) { return __float_as_uint(r.q[6].w); }

// bilinear sample of a textured kind (0 for kAffineZeroMap)
__device__ __forceinline__ float sample_kind(u32 kind, float4 q7, float4 q8, float u, float v)
{
  switch(kind)
  {
    case affine_kind(TC_TEXEL_F32, true): return affine_sample<TC_TEXEL_F32, true>(q7, q8, u, v);
    case affine_kind(TC_TEXEL_F32, false): return affine_sample<TC_TEXEL_F32, false>(q7, q8, u, v);
    case affine_kind(TC_TEXEL_F16, true): return affine_sample<TC_TEXEL_F16, true>(q7, q8, u, v);
    case affine_kind(TC_TEXEL_F16, false): return affine_sample<TC_TEXEL_F16, false>(q7, q8, u, v);
    case affine_kind(TC_TEXEL_UNORM16, true): return affine_sample<TC_TEXEL_UNORM16, true>(q7, q8, u, v);
    case affine_kind(TC_TEXEL_UNORM16, false): return affine_sample<TC_TEXEL_UNORM16, false>(q7, q8, u, v);
    default: return 0.0f;
  }
}

// Displaced vertex of a full cluster (cluster_classify.comp.glsl:457-482):
// p + normalize(n) * (bilinear(uv) * scale + offset), sampled and
// renormalised like the part vertices (Kind ~0u: resolved at run time).
template <u32 Kind>
__device__ __forceinline__ f3 full_vertex_k(f3 p, f3 n, f2 uv, const MapDesc& m, float scale, float offset)
{
  const u32 kind = Kind == ~0u ? m.kind : Kind;
  if(kind == kAffineFlat)
    return p;
  const float hraw   = sample_kind(kind, m.q7, m.q8, uv.x, uv.y);
  const float height = __fmaf_rn(hraw, scale, offset);
  const float k      = height * rsqrtf(__fmaf_rn(n.z, n.z, __fmaf_rn(n.y, n.y, n.x * n.x)));
  return fma3(k, n, p);
}

// Vertex `tableVertex` (an encoded table barycentric) of the part in `r`, for
// a record of kind Kind (~0u: any kind, resolved at run time).
template <u32 Kind>
__device__ __forceinline__ f3 affine_vertex_k(const PartAffine& r, u32 tableVertex)
{
  const float  a  = __uint2float_rn(tableVertex & 0xFFFFu) * (1.0f / 32768.0f);
  const float  b  = __uint2float_rn(tableVertex >> 16) * (1.0f / 32768.0f);
  const float4 q0 = r.q[0], q1 = r.q[1], q2 = r.q[2];
  f3           P  = {__fmaf_rn(b, q1.z, __fmaf_rn(a, q0.w, q0.x)), __fmaf_rn(b, q1.w, __fmaf_rn(a, q1.x, q0.y)),
                     __fmaf_rn(b, q2.x, __fmaf_rn(a, q1.y, q0.z))};
  const u32    kind = Kind == ~0u ? affine_kind_of(r) : Kind;
  if(kind == kAffineFlat)
    return P;
  const float4 q3 = r.q[3], q4 = r.q[4], q5 = r.q[5], q6 = r.q[6];
  const f3     N  = {__fmaf_rn(b, q3.w, __fmaf_rn(a, q3.x, q2.y)), __fmaf_rn(b, q4.x, __fmaf_rn(a, q3.y, q2.z)),
                     __fmaf_rn(b, q4.y, __fmaf_rn(a, q3.z, q2.w))};
  const float  u  = __fmaf_rn(b, q5.z, __fmaf_rn(a, q5.x, q4.z));
  const float  v  = __fmaf_rn(b, q5.w, __fmaf_rn(a, q5.y, q4.w));
  const float hraw = sample_kind(kind, r.q[7], r.q[8], u, v);
  // displace along the renormalised interpolated normal
  const float height = __fmaf_rn(hraw, q6.x, q6.y);
  const float k      = height * rsqrtf(__fmaf_rn(N.z, N.z, __fmaf_rn(N.y, N.y, N.x * N.x)));
  return fma3(k, N, P);
}

// affine_vertex_k for a record whose map, scale and offset (the same for
// every part of a chunk) are passed in registers: only q0-q5 are read from `r`.
// Same operations, so the same bits.
template <u32 Kind>
__device__ __forceinline__ f3 affine_vertex_u(const PartAffine& r, u32 tableVertex, const MapDesc& m, float scale,
                                              float offset)
{
  const float  a  = __uint2float_rn(tableVertex & 0xFFFFu) * (1.0f / 32768.0f);
  const float  b  = __uint2float_rn(tableVertex >> 16) * (1.0f / 32768.0f);
  const float4 q0 = r.q[0], q1 = r.q[1], q2 = r.q[2];
  f3           P  = {__fmaf_rn(b, q1.z, __fmaf_rn(a, q0.w, q0.x)), __fmaf_rn(b, q1.w, __fmaf_rn(a, q1.x, q0.y)),
                     __fmaf_rn(b, q2.x, __fmaf_rn(a, q1.y, q0.z))};
  const u32    kind = Kind == ~0u ? m.kind : Kind;
  if(kind == kAffineFlat)
    return P;
  const float4 q3 = r.q[3], q4 = r.q[4], q5 = r.q[5];
  const f3     N  = {__fmaf_rn(b, q3.w, __fmaf_rn(a, q3.x, q2.y)), __fmaf_rn(b, q4.x, __fmaf_rn(a, q3.y, q2.z)),
                     __fmaf_rn(b, q4.y, __fmaf_rn(a, q3.z, q2.w))};
  const float  u  = __fmaf_rn(b, q5.z, __fmaf_rn(a, q5.x, q4.z));
  const float  v  = __fmaf_rn(b, q5.w, __fmaf_rn(a, q5.y, q4.w));
  const float hraw   = sample_kind(kind, m.q7, m.q8, u, v);
  const float height = __fmaf_rn(hraw, scale, offset);
  const float k      = height * rsqrtf(__fmaf_rn(N.z, N.z, __fmaf_rn(N.y, N.y, N.x * N.x)));
  return fma3(k, N, P);
}

__device__ __forceinline__ f3 affine_vertex(const PartAffine& r, u32 tableVertex)
{
  return affine_vertex_k<~0u>(r, tableVertex);
}

__device__ __forceinline__ u32 affine_first_vertex(const PartAffine& r) { return __float_as_uint(r.q[6].z); }

}  // namespace tc

namespace tc {

// ---------------------------------------------------------------------------
// PN-triangle displacement and the ripple deformation (displacement.glsl),
// written like the CPU restatement: separate IEEE multiplies, adds and
// divisions in the shader's order.
// ---------------------------------------------------------------------------

__device__ __forceinline__ f3 add3(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 mul3(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 div3(f3 a, float s) { return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)}; }

// displacement.glsl:40-45
__device__ __forceinline__ f3 project_to_plane(f3 p, f3 plane, f3 n) { return sub3(p, mul3(n, dot3(sub3(p, plane), n))); }

// displacement.glsl:27-38 (b030 = base vertex 0, b003 = vertex 1, b300 = vertex 2)
struct BasePN
{
  f3 b030, b003, b300, b021, b012, b102, b201, b210, b120, b111;
};

// displacement.glsl:47-78 deform_setupPN; n: normalised base normals
__device__ __forceinline__ BasePN setup_pn(f3 v0, f3 v1, f3 v2, f3 n0, f3 n1, f3 n2)
{
  BasePN   b;
  b.b030         = v0;
  b.b003         = v1;
  b.b300         = v2;
  const f3 e300  = sub3(b.b003, b.b030);
  const f3 e030  = sub3(b.b300, b.b003);
  const f3 e003  = sub3(b.b030, b.b300);
  b.b021         = project_to_plane(add3(b.b030, div3(e300, 3.0f)), b.b030, n0);
  b.b012         = project_to_plane(add3(b.b030, div3(mul3(e300, 2.0f), 3.0f)), b.b003, n1);
  b.b102         = project_to_plane(add3(b.b003, div3(e030, 3.0f)), b.b003, n1);
  b.b201         = project_to_plane(add3(b.b003, div3(mul3(e030, 2.0f), 3.0f)), b.b300, n2);
  b.b210         = project_to_plane(add3(b.b300, div3(e003, 3.0f)), b.b300, n2);
  b.b120         = project_to_plane(add3(b.b300, div3(mul3(e003, 2.0f), 3.0f)), b.b030, n0);
  const f3 center = div3(add3(add3(b.b003, b.b030), b.b300), 3.0f);
  b.b111 = div3(add3(add3(add3(add3(add3(b.b021, b.b012), b.b102), b.b201), b.b210), b.b120), 6.0f);
  b.b111 = add3(b.b111, div3(sub3(b.b111, center), 2.0f));
  return b;
}

// displacement.glsl:80-104 deform_getPN (the powers as products)
__device__ __forceinline__ f3 get_pn(const BasePN& b, f3 bary)
{
  const float u = bary.x, v = bary.y, w = bary.z;
  const float u3 = u * u * u, v3 = v * v * v, w3 = w * w * w, u2 = u * u, v2 = v * v, w2 = w * w;
  f3          r = mul3(b.b300, w3);
  r             = add3(r, mul3(b.b030, u3));
  r             = add3(r, mul3(b.b003, v3));
  r             = add3(r, mul3(mul3(mul3(b.b210, 3.0f), w2), u));
  r             = add3(r, mul3(mul3(mul3(b.b120, 3.0f), w), u2));
  r             = add3(r, mul3(mul3(mul3(b.b201, 3.0f), w2), v));
  r             = add3(r, mul3(mul3(mul3(b.b021, 3.0f), u2), v));
  r             = add3(r, mul3(mul3(mul3(b.b102, 3.0f), w), v2));
  r             = add3(r, mul3(mul3(mul3(b.b012, 3.0f), u), v2));
  r             = add3(r, mul3(mul3(mul3(mul3(b.b111, 6.0f), w), u), v));
  return r;
}

// the FrameConstants terms of displacement.glsl:106-120
struct RippleParams
{
  float frequency;  // animationRippleFrequency
  float phase;      // animationState * animationRippleSpeed
  float amplitude;  // animationRippleAmplitude
  u32   enabled;
};

__device__ __forceinline__ RippleParams ripple_params(const tc_FrameConstants& view, bool enabled)
{
  return {view.animationRippleFrequency, view.animationState * view.animationRippleSpeed,
          view.animationRippleAmplitude, enabled ? 1u : 0u};
}

// displacement.glsl:106-120 rippleDeform(vertex, instance id, geometry size)
__device__ __forceinline__ f3 ripple(f3 p, u32 seed, float size, const RippleParams& rp)
{
  const float maxCoord  = fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z)));
  const float frequency = __fdiv_rn(rp.frequency, size);
  const float s         = __uint2float_rn(seed);
  const f3    wave      = {sinf((maxCoord * frequency + s) + rp.phase), cosf((maxCoord * frequency * 3.0f + s) + rp.phase),
                           sinf((maxCoord * frequency * 1.2f + s) + rp.phase)};
  const f3    dir       = normalize3({p.z, p.y, p.x});
  const float amp       = rp.amplitude * size;
  return {p.x + dir.x * (amp * wave.x), p.y + dir.y * (amp * wave.y), p.z + dir.z * (amp * wave.z)};
}

}  // namespace tc
