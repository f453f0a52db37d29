// tc_oracle.cpp — CPU oracle of the tessellated-cluster build chain.
//
// TEST INFRASTRUCTURE ONLY (see tc_oracle.h): a restatement of the reference's
// GLSL compute shaders, used by the tests and the CPU-baseline leg of the bench
// as the checker. Each function cites the reference file:line it follows
// (paths relative to the vk_tessellated_clusters checkout).
//
// Build: oracle/Makefile, with -ffp-contract=off so every a*b+c rounds twice,
// matching the CUDA kernels (compiled with -fmad=false).

#include "tc_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// small vector helpers, evaluation order fixed (left to right, no contraction)
// ---------------------------------------------------------------------------

struct f3
{
  float x, y, z;
};

inline f3 ld3(uint64_t base, uint64_t index)
{
  const float* p = (const float*)(uintptr_t)base + 3 * index;
  return {p[0], p[1], p[2]};
}

inline f3    sub3(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float len3(f3 a) { return std::sqrt(dot3(a, a)); }
inline float dist3(f3 a, f3 b) { return len3(sub3(a, b)); }
// GLSL normalize(): v * (1 / length(v)), one IEEE division then multiplies
// (GLSL leaves the exact sequence to the implementation)
inline f3 normalize3(f3 a)
{
  float r = 1.0f / len3(a);
  return {a.x * r, a.y * r, a.z * r};
}

// (M * vec4(p, 1)).xyz with column-major M
inline f3 xform_point(const float* m, f3 p)
{
  f3 r;
  r.x = ((m[0] * p.x + m[4] * p.y) + m[8] * p.z) + m[12];
  r.y = ((m[1] * p.x + m[5] * p.y) + m[9] * p.z) + m[13];
  r.z = ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14];
  return r;
}

// tessellation.glsl:191-195 tess_interpolate (precise)
inline f3 interp3(const f3 b[3], f3 w)
{
  f3 r;
  r.x = (b[0].x * w.x + b[1].x * w.y) + b[2].x * w.z;
  r.y = (b[0].y * w.x + b[1].y * w.y) + b[2].y * w.z;
  r.z = (b[0].z * w.x + b[1].z * w.y) + b[2].z * w.z;
  return r;
}

struct f2
{
  float x, y;
};
// tessellation.glsl:197-201
inline f2 interp2(const f2 b[3], f3 w)
{
  f2 r;
  r.x = (b[0].x * w.x + b[1].x * w.y) + b[2].x * w.z;
  r.y = (b[0].y * w.x + b[1].y * w.y) + b[2].y * w.z;
  return r;
}

template <class T>
inline T* P(uint64_t a)
{
  return (T*)(uintptr_t)a;
}

// ---------------------------------------------------------------------------
// tessellation.glsl
// ---------------------------------------------------------------------------

// tessellation.glsl:48-59
uint32_t encodeBary(f3 wuv)
{
  uint32_t ix = (uint32_t)(wuv.x * 32768.0f + 0.5f);
  uint32_t iy = (uint32_t)(wuv.y * 32768.0f + 0.5f);
  uint32_t iz = (uint32_t)(wuv.z * 32768.0f + 0.5f);
  if(ix > std::max(iy, iz))
    ix = 32768u - iy - iz;
  else if(iy > iz)
    iy = 32768u - ix - iz;
  else
    iz = 32768u - ix - iy;
  return iy | (iz << 16);
}

// tessellation.glsl:66-76
f3 decodeBary(uint32_t vtx)
{
  f3 w;
  w.y = float(vtx & 0xFFFFu) / 32768.0f;
  w.z = float(vtx >> 16) / 32768.0f;
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

inline uint32_t roundClampFactor(float e, float spl, const FactorParams& fp)
{
  float f = std::nearbyint(((e * spl) * fp.viewportH) * fp.tessRate);
  f       = std::min(std::max(f, 1.0f), 32768.0f);
  return (uint32_t)f;
}

// tessellation.glsl:78-99
void tessFactors(f3 a, f3 b, f3 c, const FactorParams& fp, uint32_t out[3])
{
  float da = dist3(a, fp.viewPos);
  float db = dist3(b, fp.viewPos);
  float dc = dist3(c, fp.viewPos);
  float sx = 1.0f / std::max(fp.nearPlane, std::min(da, db));
  float sy = 1.0f / std::max(fp.nearPlane, std::min(db, dc));
  float sz = 1.0f / std::max(fp.nearPlane, std::min(dc, da));
  float ex = dist3(a, b);
  float ey = dist3(b, c);
  float ez = dist3(c, a);
  out[0]   = roundClampFactor(ex, sx, fp);
  out[1]   = roundClampFactor(ey, sy, fp);
  out[2]   = roundClampFactor(ez, sz, fp);
}

// tessellation.glsl:101-104
inline uint32_t splitFactor1(uint32_t f, uint32_t sf) { return std::min((f + TC_TESSTABLE_SIZE - 1) / TC_TESSTABLE_SIZE, sf); }

// tessellation.glsl:119-144
uint32_t getConfig(uint32_t f[3], uint32_t tv[3])
{
  uint32_t m = std::max(std::max(f[0], f[1]), f[2]);
  if(m == f[1])
  {
    uint32_t a = f[0], b = f[1], c = f[2];
    f[0] = b, f[1] = c, f[2] = a;
    a = tv[0], b = tv[1], c = tv[2];
    tv[0] = b, tv[1] = c, tv[2] = a;
  }
  else if(m == f[2])
  {
    uint32_t a = f[0], b = f[1], c = f[2];
    f[0] = c, f[1] = a, f[2] = b;
    a = tv[0], b = tv[1], c = tv[2];
    tv[0] = c, tv[1] = a, tv[2] = b;
  }
  const uint32_t L   = TC_TESSTABLE_LOOKUP_SIZE;
  uint32_t       idx = f[0] + f[1] * L + f[2] * L * L - (1 + L + L * L);
  if(f[2] > f[1])
    idx |= 1u << 15;
  return idx;
}

inline uint32_t cfgIndex(uint32_t cfg) { return cfg & ~(1u << 15); }
inline bool     cfgFlipped(uint32_t cfg) { return (cfg & (1u << 15)) != 0; }

// tessellation.glsl:165-176
inline void cfgTriangle(const tco_table* t, uint32_t cfg, uint32_t tri, uint32_t out[3])
{
  const tc_TessTableEntry& e = t->entries[cfgIndex(cfg)];
  uint32_t                 p = t->triangles[e.firstTriangle + tri];
  out[0]                     = p & 0xFF;
  out[1]                     = (p >> 8) & 0xFF;
  out[2]                     = (p >> 16) & 0xFF;
  if(cfgFlipped(cfg))
    std::swap(out[1], out[2]);
}

// tessellation.glsl:178-189
inline f3 cfgVertex(const tco_table* t, uint32_t cfg, uint32_t vert)
{
  const tc_TessTableEntry& e = t->entries[cfgIndex(cfg)];
  f3                       w = decodeBary(t->vertices[e.firstVertex + vert]);
  if(cfgFlipped(cfg))
    std::swap(w.x, w.y);
  return w;
}

// ---------------------------------------------------------------------------
// displacement sampling: bilinear, mip 0, REPEAT, texel centres at i + 0.5
// ---------------------------------------------------------------------------

float halfToFloat(uint16_t h)
{
  uint32_t sign = (uint32_t)(h >> 15) << 31;
  uint32_t exp  = (h >> 10) & 0x1F;
  uint32_t man  = h & 0x3FF;
  uint32_t bits;
  if(exp == 0)
  {
    if(man == 0)
      bits = sign;
    else
    {
      // subnormal: normalise
      int e = -1;
      do
      {
        man <<= 1;
        e++;
      } while((man & 0x400) == 0);
      man &= 0x3FF;
      bits = sign | ((uint32_t)(127 - 15 - e) << 23) | (man << 13);
    }
  }
  else if(exp == 31)
    bits = sign | 0x7F800000u | (man << 13);
  else
    bits = sign | ((exp + 127 - 15) << 23) | (man << 13);
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

inline float texel(const tc_DisplacementTexture& tx, int x, int y)
{
  size_t i = (size_t)y * tx.width + (size_t)x;
  switch(tx.format)
  {
    case TC_TEXEL_F16:
      return halfToFloat(P<const uint16_t>(tx.texels)[i]);
    case TC_TEXEL_UNORM16:
      return float(P<const uint16_t>(tx.texels)[i]) / 65535.0f;
    default:
      return P<const float>(tx.texels)[i];
  }
}

inline int wrapi(int i, int n)
{
  int r = i % n;
  return r < 0 ? r + n : r;
}

struct BilinearTaps
{
  int   x0, x1, y0, y1;
  float fx, fy;
};

inline BilinearTaps bilinearTaps(const tc_DisplacementTexture& tx, f2 uv)
{
  float        x  = uv.x * (float)tx.width - 0.5f;
  float        y  = uv.y * (float)tx.height - 0.5f;
  float        xf = std::floor(x);
  float        yf = std::floor(y);
  BilinearTaps b;
  b.fx = x - xf;
  b.fy = y - yf;
  int ix = (int)xf, iy = (int)yf;
  b.x0 = wrapi(ix, (int)tx.width);
  b.x1 = wrapi(ix + 1, (int)tx.width);
  b.y0 = wrapi(iy, (int)tx.height);
  b.y1 = wrapi(iy + 1, (int)tx.height);
  return b;
}

float sampleBilinear(const tc_DisplacementTexture& tx, f2 uv)
{
  if(tx.width == 0 || tx.height == 0)
    return 0.0f;
  BilinearTaps b   = bilinearTaps(tx, uv);
  float        t00 = texel(tx, b.x0, b.y0);
  float        t10 = texel(tx, b.x1, b.y0);
  float        t01 = texel(tx, b.x0, b.y1);
  float        t11 = texel(tx, b.x1, b.y1);
  float        gx  = 1.0f - b.fx;
  float        top = gx * t00 + b.fx * t10;
  float        bot = gx * t01 + b.fx * t11;
  return (1.0f - b.fy) * top + b.fy * bot;
}

// cluster_classify.comp.glsl:471-478 / triangle_tess_template_instantiate.comp.glsl:356-365
inline const tc_DisplacementTexture* instanceTexture(const tc_frame_args* a, const tc_RenderInstance& inst)
{
  if(a->numTextures == 0 || a->textures == 0 || inst.displacementIndex < 0 || (uint32_t)inst.displacementIndex >= a->numTextures)
    return nullptr;
  return &P<const tc_DisplacementTexture>(a->textures)[inst.displacementIndex];
}

inline f3 displace(f3 pos, f3 normal, f2 uv, const tc_DisplacementTexture* tx, const tc_RenderInstance& inst,
                   const tc_FrameConstants& view)
{
  float h = sampleBilinear(*tx, uv);
  h       = ((h * inst.displacementScale) * view.displacementScale + inst.displacementOffset) + view.displacementOffset;
  f3 n    = normalize3(normal);
  return {pos.x + n.x * h, pos.y + n.y * h, pos.z + n.z * h};
}

// displacement.glsl:47-78 deform_setupPN: the PN triangle's ten control
// points from the base positions and (normalised) normals, with the shader's
// corner naming (b030 = vertex 0, b003 = vertex 1, b300 = vertex 2)
struct BasePN
{
  f3 b030, b003, b300, b021, b012, b102, b201, b210, b120, b111;
};

inline f3 add3(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline f3 mul3(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline f3 div3(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }

// displacement.glsl:40-45
inline f3 projectToPlane(f3 p, f3 plane, f3 n) { return sub3(p, mul3(n, dot3(sub3(p, plane), n))); }

inline BasePN setupPN(const f3 v[3], const f3 n[3])
{
  BasePN b;
  b.b030         = v[0];
  b.b003         = v[1];
  b.b300         = v[2];
  const f3 e300  = sub3(b.b003, b.b030);
  const f3 e030  = sub3(b.b300, b.b003);
  const f3 e003  = sub3(b.b030, b.b300);
  b.b021         = add3(b.b030, div3(e300, 3.0f));
  b.b012         = add3(b.b030, div3(mul3(e300, 2.0f), 3.0f));
  b.b102         = add3(b.b003, div3(e030, 3.0f));
  b.b201         = add3(b.b003, div3(mul3(e030, 2.0f), 3.0f));
  b.b210         = add3(b.b300, div3(e003, 3.0f));
  b.b120         = add3(b.b300, div3(mul3(e003, 2.0f), 3.0f));
  b.b021         = projectToPlane(b.b021, b.b030, n[0]);
  b.b012         = projectToPlane(b.b012, b.b003, n[1]);
  b.b102         = projectToPlane(b.b102, b.b003, n[1]);
  b.b201         = projectToPlane(b.b201, b.b300, n[2]);
  b.b210         = projectToPlane(b.b210, b.b300, n[2]);
  b.b120         = projectToPlane(b.b120, b.b030, n[0]);
  const f3 center = div3(add3(add3(b.b003, b.b030), b.b300), 3.0f);
  b.b111 = div3(add3(add3(add3(add3(add3(b.b021, b.b012), b.b102), b.b201), b.b210), b.b120), 6.0f);
  b.b111 = add3(b.b111, div3(sub3(b.b111, center), 2.0f));
  return b;
}

// displacement.glsl:80-104 deform_getPN (pow(x, 2 / 3) as products), terms
// summed left to right, scalar factors applied left to right
inline f3 getPN(const BasePN& b, f3 bary)
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

// displacement.glsl:106-120 rippleDeform(vertex, instance id, geometry size)
inline f3 ripple(f3 p, uint32_t seed, float size, const tc_FrameConstants& view)
{
  const float maxCoord  = std::max(std::fabs(p.x), std::max(std::fabs(p.y), std::fabs(p.z)));
  const float frequency = view.animationRippleFrequency / size;
  const float phase     = view.animationState * view.animationRippleSpeed;
  const float s         = float(seed);
  const f3    wave      = {std::sin((maxCoord * frequency + s) + phase), std::cos((maxCoord * frequency * 3.0f + s) + phase),
                           std::sin((maxCoord * frequency * 1.2f + s) + phase)};
  const f3    dir       = normalize3({p.z, p.y, p.x});
  const float amp       = view.animationRippleAmplitude * size;
  return {p.x + dir.x * (amp * wave.x), p.y + dir.y * (amp * wave.y), p.z + dir.z * (amp * wave.z)};
}

// ---------------------------------------------------------------------------
// threading
// ---------------------------------------------------------------------------

template <class F>
void parallelFor(size_t n, int threads, F&& fn)
{
  if(threads <= 1 || n < 64)
  {
    fn(size_t(0), n);
    return;
  }
  size_t                   nt    = std::min<size_t>((size_t)threads, (n + 63) / 64);
  size_t                   chunk = (n + nt - 1) / nt;
  std::vector<std::thread> pool;
  for(size_t t = 0; t < nt; t++)
  {
    size_t b = t * chunk, e = std::min(n, b + chunk);
    if(b >= e)
      break;
    pool.emplace_back([&fn, b, e]() { fn(b, e); });
  }
  for(auto& th : pool)
    th.join();
}

struct Ctx
{
  const tc_frame_args*     a;
  tc_SceneBuilding*        b;
  tc_Readback*             rb;
  const tc_FrameConstants* view;
  const tc_FrameConstants* viewLast;
  const tc_RenderInstance* inst;
  FactorParams             fp;
  uint64_t                 maxDataBytes;

  explicit Ctx(const tc_frame_args* args)
  {
    a            = args;
    b            = P<tc_SceneBuilding>(args->build);
    rb           = P<tc_Readback>(args->readback);
    view         = P<const tc_FrameConstants>(args->view);
    viewLast     = P<const tc_FrameConstants>(args->viewLast);
    inst         = P<const tc_RenderInstance>(args->instances);
    fp.viewPos   = {b->viewPos.x, b->viewPos.y, b->viewPos.z};
    fp.nearPlane = view->nearPlane;
    fp.viewportH = view->viewportf.y;
    fp.tessRate  = view->tessRate;
    maxDataBytes = uint64_t(args->caps.maxGeneratedClusterMegs) * 1024 * 1024;
  }
};

uint32_t clampSplitFactor(uint32_t sf) { return std::max(2u, std::min(sf, TC_TESSTABLE_SIZE)); }

// ---------------------------------------------------------------------------
// culling.glsl
// ---------------------------------------------------------------------------

void matMul(const float* A, const float* B, float* C)
{
  // C = A * B (column-major): C[c][r] = sum_k A[k][r] * B[c][k], summed k = 0..3 in order
  for(int c = 0; c < 4; c++)
    for(int r = 0; r < 4; r++)
      C[c * 4 + r] = ((A[0 * 4 + r] * B[c * 4 + 0] + A[1 * 4 + r] * B[c * 4 + 1]) + A[2 * 4 + r] * B[c * 4 + 2])
                     + A[3 * 4 + r] * B[c * 4 + 3];
}

struct Clip
{
  float x, y, z, w;
};

// culling.glsl:50-90
bool intersectFrustum(f3 lo, f3 hi, const float* world, const tc_FrameConstants& vl, Clip& omin, Clip& omax, bool& ovalid)
{
  float wvp[16];
  matMul(vl.viewProjMatrix.m, world, wvp);
  const float eps    = 1.2e-07f;
  uint32_t    bits   = 0x7F;
  bool        valid  = true;
  Clip        cmin   = {0, 0, 0, 0}, cmax = {0, 0, 0, 0};
  for(int n = 0; n < 8; n++)
  {
    float p[4] = {(n & 1) ? hi.x : lo.x, (n & 2) ? hi.y : lo.y, (n & 4) ? hi.z : lo.z, 1.0f};
    float h[4];
    for(int r = 0; r < 4; r++)
      h[r] = ((wvp[r] * p[0] + wvp[4 + r] * p[1]) + wvp[8 + r] * p[2]) + wvp[12 + r] * p[3];
    bool     v  = !(-eps < h[3] && h[3] < eps);
    float    aw = std::fabs(h[3]);
    Clip     c  = {h[0] / aw, h[1] / aw, h[2] / aw, h[3]};
    uint32_t cb = 0;
    cb |= h[0] < -h[3] ? 1 : 0;
    cb |= h[0] > h[3] ? 2 : 0;
    cb |= h[1] < -h[3] ? 4 : 0;
    cb |= h[1] > h[3] ? 8 : 0;
    cb |= h[2] < 0 ? 16 : 0;
    cb |= h[2] > h[3] ? 32 : 0;
    cb |= h[3] <= 0 ? 64 : 0;
    if(n == 0)
    {
      bits = cb;
      cmin = c;
      cmax = c;
      valid = v;
    }
    else
    {
      bits &= cb;
      cmin = {std::min(cmin.x, c.x), std::min(cmin.y, c.y), std::min(cmin.z, c.z), std::min(cmin.w, c.w)};
      cmax = {std::max(cmax.x, c.x), std::max(cmax.y, c.y), std::max(cmax.z, c.z), std::max(cmax.w, c.w)};
      valid = valid && v;
    }
  }
  ovalid = valid;
  omin   = {std::min(std::max(cmin.x, -1.0f), 1.0f), std::min(std::max(cmin.y, -1.0f), 1.0f), cmin.z, cmin.w};
  omax   = {std::min(std::max(cmax.x, -1.0f), 1.0f), std::min(std::max(cmax.y, -1.0f), 1.0f), cmax.z, cmax.w};
  return bits == 0;
}

// culling.glsl:30-35
bool intersectSize(const Clip& cmin, const Clip& cmax, const tc_FrameConstants& vl)
{
  float rx = cmax.x - cmin.x, ry = cmax.y - cmin.y;
  float tx = 2.0f / vl.viewportf.x, ty = 2.0f / vl.viewportf.y;
  return rx > tx || ry > ty;
}

// culling.glsl:94-113: the HiZ test needs last frame's depth pyramid, which a
// headless build does not have; it always passes.
bool intersectHiz(const Clip&, const Clip&) { return true; }

}  // namespace

// ===========================================================================
// exported API
// ===========================================================================

extern "C" {

// src/tessellation_table.cpp:36-83
int tco_table_init(tco_table* t, const uint32_t* vertices, uint32_t numVertices, const uint32_t* triangles,
                   uint32_t numTriangles, const uint16_t* configs, uint32_t numConfigs, uint32_t maxEdgeSegments)
{
  if(maxEdgeSegments != TC_TESSTABLE_SIZE)
    return 1;
  std::memset(t, 0, sizeof(*t));
  t->vertices     = vertices;
  t->triangles    = triangles;
  t->numVertices  = numVertices;
  t->numTriangles = numTriangles;
  const uint32_t L = TC_TESSTABLE_LOOKUP_SIZE;
  auto lookup = [&](uint32_t x, uint32_t y, uint32_t z) { return x + y * L + z * L * L - (1 + L + L * L); };
  uint32_t ci = 0;
  for(uint32_t x = 1; x <= maxEdgeSegments; x++)
    for(uint32_t y = 1; y <= x; y++)
      for(uint32_t z = 1; z <= y; z++, ci++)
      {
        if(ci >= numConfigs)
          return 2;
        tc_TessTableEntry e = {configs[ci * 4 + 0], configs[ci * 4 + 1], configs[ci * 4 + 2], configs[ci * 4 + 3]};
        t->entries[lookup(x, y, z)] = e;
        if(z != y && x > 1)
          t->entries[lookup(x, z, y)] = e;
        t->maxTriangles = std::max(t->maxTriangles, (uint32_t)e.numTriangles);
        t->maxVertices  = std::max(t->maxVertices, (uint32_t)e.numVertices);
      }
  return ci == numConfigs ? 0 : 3;
}

uint32_t tco_encode_barycentrics(float w, float u, float v) { return encodeBary({w, u, v}); }

void tco_decode_barycentrics(uint32_t enc, float* out3)
{
  f3 w    = decodeBary(enc);
  out3[0] = w.x;
  out3[1] = w.y;
  out3[2] = w.z;
}

void tco_tess_factors(const float* a, const float* b, const float* c, const float* viewPos, float nearPlane,
                      float viewportH, float tessRate, uint32_t* out3)
{
  FactorParams fp = {{viewPos[0], viewPos[1], viewPos[2]}, nearPlane, viewportH, tessRate};
  tessFactors({a[0], a[1], a[2]}, {b[0], b[1], b[2]}, {c[0], c[1], c[2]}, fp, out3);
}

uint32_t tco_get_config(const uint32_t* factors3, uint32_t* triangleVertices3)
{
  uint32_t f[3] = {factors3[0], factors3[1], factors3[2]};
  return getConfig(f, triangleVertices3);
}

uint32_t tco_split_factor(uint32_t factor, uint32_t splitFactor) { return splitFactor1(factor, clampSplitFactor(splitFactor)); }

void tco_config_triangle(const tco_table* t, uint32_t cfg, uint32_t tri, uint32_t* out3) { cfgTriangle(t, cfg, tri, out3); }

void tco_config_vertex(const tco_table* t, uint32_t cfg, uint32_t vert, float* out3)
{
  const f3 w = cfgVertex(t, cfg, vert);
  out3[0] = w.x, out3[1] = w.y, out3[2] = w.z;
}

void tco_interpolate3(const float* base9, const float* wuv, float* out3)
{
  const f3 b[3] = {{base9[0], base9[1], base9[2]}, {base9[3], base9[4], base9[5]}, {base9[6], base9[7], base9[8]}};
  const f3 r    = interp3(b, {wuv[0], wuv[1], wuv[2]});
  out3[0] = r.x, out3[1] = r.y, out3[2] = r.z;
}

void tco_pn_position(const float* verts9, const float* normals9, const float* bary3, float* out3)
{
  const f3 v[3] = {{verts9[0], verts9[1], verts9[2]}, {verts9[3], verts9[4], verts9[5]}, {verts9[6], verts9[7], verts9[8]}};
  const f3 n[3] = {{normals9[0], normals9[1], normals9[2]},
                   {normals9[3], normals9[4], normals9[5]},
                   {normals9[6], normals9[7], normals9[8]}};
  const f3 r    = getPN(setupPN(v, n), {bary3[0], bary3[1], bary3[2]});
  out3[0] = r.x, out3[1] = r.y, out3[2] = r.z;
}

void tco_ripple(const float* p3, uint32_t seed, float geometrySize, const tc_FrameConstants* view, float* out3)
{
  const f3 r = ripple({p3[0], p3[1], p3[2]}, seed, geometrySize, *view);
  out3[0] = r.x, out3[1] = r.y, out3[2] = r.z;
}

int tco_intersect_frustum(const float* lo3, const float* hi3, const float* world16, const tc_FrameConstants* viewLast,
                          float* clipMin4, float* clipMax4, int* clipValid)
{
  Clip       cmin, cmax;
  bool       valid = false;
  const bool in    = intersectFrustum({lo3[0], lo3[1], lo3[2]}, {hi3[0], hi3[1], hi3[2]}, world16, *viewLast, cmin, cmax, valid);
  clipMin4[0] = cmin.x, clipMin4[1] = cmin.y, clipMin4[2] = cmin.z, clipMin4[3] = cmin.w;
  clipMax4[0] = cmax.x, clipMax4[1] = cmax.y, clipMax4[2] = cmax.z, clipMax4[3] = cmax.w;
  *clipValid  = valid ? 1 : 0;
  return in ? 1 : 0;
}

int tco_intersect_size(const float* clipMin4, const float* clipMax4, const tc_FrameConstants* viewLast)
{
  const Clip cmin = {clipMin4[0], clipMin4[1], clipMin4[2], clipMin4[3]};
  const Clip cmax = {clipMax4[0], clipMax4[1], clipMax4[2], clipMax4[3]};
  return intersectSize(cmin, cmax, *viewLast) ? 1 : 0;
}

// src/renderer_raytrace_clusters_tess.cpp:516-519
uint32_t tco_split_pass_count(uint32_t splitFactor)
{
  uint32_t sf = clampSplitFactor(splitFactor);
  uint32_t n = 0, coord = TC_TESSTABLE_COORD_MAX;
  while(coord > sf)
  {
    coord /= sf;
    n++;
  }
  return n;
}

// src/renderer_raytrace_clusters_tess.cpp:412-419 (per-frame counter reset via the host
// copy of SceneBuilding, readback clear, split buffer fill with ~0)
void tco_frame_begin(const tc_frame_args* a)
{
  Ctx c(a);
  tc_SceneBuilding*        b  = c.b;
  const tc_FrameConstants* vp = (a->flags & TC_FLAG_FREEZE_VIEWPOS) ? c.viewLast : c.view;
  b->viewPos                  = {vp->viewPos.x, vp->viewPos.y, vp->viewPos.z};
  b->numRenderInstances       = a->numInstances;
  b->visibleClusterCounter    = 0;
  b->fullClusterCounter       = 0;
  b->partTriangleCounter      = 0;
  b->dualPartTriangleCounter  = 0;
  b->splitTriangleCounter     = 0;
  b->splitReadCounter         = 0;
  b->splitWriteCounter        = 0;
  b->splitPass                = 0;
  b->splitPassStart           = 0;
  b->splitPassEnd             = 0;
  b->genVertexCounter         = 0;
  b->genClusterCounter        = 0;
  b->genClusterDataCounter    = 0;
  b->dispatchClassify         = {0, 0, 0};
  b->dispatchTriangleSplit    = {0, 0, 0};
  b->drawFullClusters         = {0, 0};
  b->drawPartTriangles        = {0, 0};
  b->dispatchClusterInstantiate  = {0, 0, 0};
  b->dispatchTriangleInstantiate = {0, 0, 0};
  b->dispatchBlasTempInsert      = {0, 0, 0};
  b->dispatchBlasTransInsert     = {0, 0, 0};
  b->blasClusterCounter          = 0;
  b->tempInstantiateCounter      = 0;
  b->transBuildCounter           = 0;
  std::memset(c.rb, 0, sizeof(tc_Readback));
  if(b->splitTriangles)
    std::memset(P<void>(b->splitTriangles), 0xFF, sizeof(tc_TessTriangleInfo) * (size_t)a->caps.maxSplitTriangles);
}

// shaders/instances_classify.comp.glsl:102-128
void tco_instances_classify(const tc_frame_args* a)
{
  Ctx c(a);
  for(uint32_t i = 0; i < a->numInstances; i++)
  {
    const tc_RenderInstance& in = c.inst[i];
    Clip                     cmin, cmax;
    bool                     cvalid;
    bool inFrustum = intersectFrustum({in.geoLo.x, in.geoLo.y, in.geoLo.z}, {in.geoHi.x, in.geoHi.y, in.geoHi.z},
                                      in.worldMatrix.m, *c.viewLast, cmin, cmax, cvalid);
    bool visible = inFrustum && (!cvalid || (intersectSize(cmin, cmax, *c.viewLast) && intersectHiz(cmin, cmax)));
    P<uint32_t>(c.b->instanceStates)[i] = (inFrustum ? TC_INSTANCE_FRUSTUM_BIT : 0) | (visible ? TC_INSTANCE_VISIBLE_BIT : 0);
    P<tc_BlasBuildInfo>(c.b->blasBuildInfos)[i].clusterReferencesCount = 0;
  }
}

// shaders/clusters_cull.comp.glsl:112-161, for every instance in order
// (src/renderer_raytrace_clusters_tess.cpp:454-460)
void tco_clusters_cull(const tc_frame_args* a)
{
  Ctx              c(a);
  const bool       rasterCull = (a->flags & TC_FLAG_RASTER_CULL) && (a->flags & TC_FLAG_CULLING);
  tc_ClusterInfo*  vis        = P<tc_ClusterInfo>(c.b->visibleClusters);
  const uint32_t*  states     = P<const uint32_t>(c.b->instanceStates);
  for(uint32_t i = 0; i < a->numInstances; i++)
  {
    const tc_RenderInstance& in = c.inst[i];
    for(uint32_t k = 0; k < in.numClusters; k++)
    {
      bool visible = true;
      if(rasterCull)
      {
        const tc_BBox& bb = P<const tc_BBox>(in.clusterBboxes)[k];
        Clip           cmin, cmax;
        bool           cvalid;
        if((states[i] & TC_INSTANCE_VISIBLE_BIT) == 0)
          visible = false;
        visible = visible
                  && intersectFrustum({bb.lo.x, bb.lo.y, bb.lo.z}, {bb.hi.x, bb.hi.y, bb.hi.z}, in.worldMatrix.m,
                                      *c.viewLast, cmin, cmax, cvalid);
        visible = visible && (!cvalid || (intersectSize(cmin, cmax, *c.viewLast) && intersectHiz(cmin, cmax)));
      }
      if(visible)
      {
        uint32_t off = c.b->visibleClusterCounter++;
        if(off < a->caps.maxVisibleClusters)
          vis[off] = {i, k};
      }
    }
  }
}

// shaders/build_setup.comp.glsl:102-265 (RT target, multipass split; with
// transient builds :193-265 read the two-sided part counter and the transient
// build count)
void tco_build_setup(const tc_frame_args* a, uint32_t mode)
{
  Ctx               c(a);
  const bool        trans = (a->flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X)) != 0;
  tc_SceneBuilding* b  = c.b;
  tc_Readback*      rb = c.rb;
  const tc_caps&    k  = a->caps;
  switch(mode)
  {
    case TC_BUILD_SETUP_CLASSIFY:
    {
      uint32_t counter       = b->visibleClusterCounter;
      rb->numVisibleClusters = counter;
      counter                = std::min(counter, k.maxVisibleClusters);
      b->visibleClusterCounter = counter;
      b->dispatchClassify      = {counter, 1, 1};
      break;
    }
    case TC_BUILD_SETUP_DRAW_TESS:
    {
      uint32_t full = b->fullClusterCounter, part = b->partTriangleCounter;
      rb->numFullClusters   = full;
      rb->numPartTriangles  = part;
      rb->numSplitTriangles = b->splitWriteCounter;
      full                  = std::min(full, k.maxVisibleClusters);
      part                  = std::min(part, k.maxPartTriangles);
      b->drawFullClusters   = {full, 0};
      b->drawPartTriangles  = {(part + 31) / 32, 0};
      rb->numBlasClusters   = full;
      break;
    }
    case TC_BUILD_SETUP_SPLIT:
    {
      uint32_t count = (uint32_t)std::min<int64_t>((int64_t)b->splitTriangleCounter, (int64_t)k.maxSplitTriangles);
      b->splitWriteCounter    = count;
      b->splitTriangleCounter = (int32_t)count;
      b->splitPassStart       = 0;
      b->splitPassEnd         = count;
      b->dispatchTriangleSplit = {(count + 63) / 64, 1, 1};
      break;
    }
    case TC_BUILD_SETUP_SPLIT_PASS:
    {
      uint32_t pass    = b->splitPass + 1;
      b->splitPass     = pass;
      uint32_t start   = std::min(b->splitPassEnd, k.maxSplitTriangles);
      uint32_t end     = std::min(b->splitWriteCounter, k.maxSplitTriangles);
      b->splitPassStart = start;
      b->splitPassEnd   = end;
      b->dispatchTriangleSplit = {(end - start + 63) / 64, 1, 1};
      break;
    }
    case TC_BUILD_SETUP_BUILD_BLAS:
    {
      uint32_t temp               = b->tempInstantiateCounter;
      uint32_t tr                 = trans ? b->transBuildCounter : 0u;
      rb->numBlasClusters         = temp + tr;
      rb->numTransBuilds          = tr;
      rb->numTempInstantiations   = temp;
      rb->numGenDatas             = b->genClusterDataCounter;
      rb->numGenVertices          = b->genVertexCounter;
      rb->numBlasReservedSizes    = b->numBlasReservedSizes;
      temp                        = std::min(k.maxGeneratedClusters, temp);
      b->tempInstantiateCounter   = temp;
      rb->numActualTempInstantiations = temp;
      b->dispatchBlasTempInsert   = {(temp + 63) / 64, 1, 1};
      if(trans)
      {
        tr                          = std::min(k.maxGeneratedClusters, temp + tr) - temp;
        b->transBuildCounter        = tr;
        rb->numActualTransBuilds    = tr;
        b->dispatchBlasTransInsert  = {(tr + 63) / 64, 1, 1};
      }
      break;
    }
    case TC_BUILD_SETUP_INSTANTIATE_TESS:
    {
      uint32_t part           = b->partTriangleCounter;
      rb->numSplitTriangles   = b->splitWriteCounter;
      if(trans)
      {
        // requests from both ends; partTriangleCounter is the written front's end
        const uint32_t lo = (uint32_t)b->dualPartTriangleCounter, hi = (uint32_t)(b->dualPartTriangleCounter >> 32);
        rb->numPartTriangles      = lo + hi;
        rb->numTransPartTriangles = hi;
      }
      else
        rb->numPartTriangles = part;
      part                    = std::min(part, k.maxPartTriangles);
      b->partTriangleCounter  = part;
      b->dispatchTriangleInstantiate = {(part + 31) / 32, 1, 1};
      break;
    }
    default:
      break;
  }
}

}  // extern "C"

namespace {

// per visible cluster: its triangles' edge factors and how many need no tessellation
struct ClassifyRec
{
  uint32_t simple;
  uint32_t numTriangles;
  uint32_t factors[64][3];
};

void classifyTransient(const tco_table* t, const tc_frame_args* a, std::vector<ClassifyRec>& recs, int numThreads);

}  // namespace

extern "C" {

// shaders/cluster_classify.comp.glsl:150-666 (RT target, plain path)
void tco_cluster_classify(const tco_table* t, const tc_frame_args* a, int numThreads)
{
  Ctx                  c(a);
  tc_SceneBuilding*    b     = c.b;
  const uint32_t       nvis  = b->visibleClusterCounter;
  const tc_ClusterInfo* vis  = P<const tc_ClusterInfo>(b->visibleClusters);
  const uint32_t*      states = P<const uint32_t>(b->instanceStates);
  const bool           culling = (a->flags & TC_FLAG_CULLING) != 0;

  using Rec = ClassifyRec;
  std::vector<Rec> recs(nvis);

  // phase 1: factors (parallel)
  parallelFor(nvis, numThreads, [&](size_t lo, size_t hi) {
    for(size_t v = lo; v < hi; v++)
    {
      const tc_ClusterInfo&    ci = vis[v];
      const tc_RenderInstance& in = c.inst[ci.instanceID];
      const tc_Cluster&        cl = P<const tc_Cluster>(in.clusters)[ci.clusterID];
      Rec&                     r  = recs[v];
      r.numTriangles              = cl.numTriangles;
      r.simple                    = 0;
      if(culling && (states[ci.instanceID] & TC_INSTANCE_VISIBLE_BIT) == 0)
      {
        r.simple = cl.numTriangles;
        continue;
      }
      const uint8_t* lt = P<const uint8_t>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      for(uint32_t tri = 0; tri < cl.numTriangles && tri < 64; tri++)
      {
        f3 w[3];
        for(int k = 0; k < 3; k++)
          w[k] = xform_point(in.worldMatrix.m, ld3(in.positions, cl.firstLocalVertex + lt[tri * 3 + k]));
        tessFactors(w[0], w[1], w[2], c.fp, r.factors[tri]);
        uint32_t m = std::max(std::max(r.factors[tri][0], r.factors[tri][1]), r.factors[tri][2]);
        r.simple += m == 1 ? 1 : 0;
      }
    }
  });

  if(a->flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
  {
    classifyTransient(t, a, recs, numThreads);
    return;
  }

  // phase 2: serial allocation in canonical order
  struct Alloc
  {
    uint32_t vertexOffset;  // ~0 = rejected / not full
    uint32_t tempOffset;
    uint64_t dataOffset;
  };
  std::vector<Alloc> alloc(nvis);
  struct TriOut
  {
    uint32_t cluster, tri, offset;
    bool     split;
  };
  std::vector<TriOut> triOut;
  const tc_caps&      k = a->caps;
  for(uint32_t v = 0; v < nvis; v++)
  {
    const tc_ClusterInfo&    ci = vis[v];
    const tc_RenderInstance& in = c.inst[ci.instanceID];
    const tc_Cluster&        cl = P<const tc_Cluster>(in.clusters)[ci.clusterID];
    Rec&                     r  = recs[v];
    alloc[v].vertexOffset       = ~0u;
    if(r.simple == r.numTriangles)
    {
      c.rb->numFullClusters += 1;
      uint32_t genOffset    = b->genClusterCounter++;
      uint64_t dataSize     = P<const uint32_t>(in.clusterTemplateInstantiatonSizes)[ci.clusterID];
      uint64_t dataOffset   = b->genClusterDataCounter;
      b->genClusterDataCounter += dataSize;
      uint32_t vertexOffset = b->genVertexCounter;
      b->genVertexCounter += cl.numVertices;
      if((uint64_t)vertexOffset + cl.numVertices > k.maxGeneratedVertices || genOffset + 1 > k.maxGeneratedClusters
         || dataOffset + dataSize > c.maxDataBytes)
        continue;
      uint32_t tempOffset   = b->tempInstantiateCounter++;
      alloc[v]              = {vertexOffset, tempOffset, dataOffset};
      tc_TemplateInstantiateInfo ti;
      ti.clusterIdOffset        = 0;
      ti.geometryIndexOffset    = 0;
      ti.clusterTemplateAddress = P<const uint64_t>(in.clusterTemplateAdresses)[ci.clusterID];
      ti.vertexBufferAddress    = b->genVertices + uint64_t(vertexOffset) * 12;
      ti.vertexBufferStride     = 12;
      P<tc_TemplateInstantiateInfo>(b->tempInstantiations)[tempOffset] = ti;
      P<uint32_t>(b->tempInstanceIDs)[tempOffset]                      = ci.instanceID;
      P<uint64_t>(b->tempClusterAddresses)[tempOffset]                 = b->genClusterData + dataOffset;
      if((a->flags & TC_FLAG_WRITE_FULLCLUSTERS) && b->fullClusters)
        P<tc_ClusterInfo>(b->fullClusters)[tempOffset] = ci;
      P<tc_BlasBuildInfo>(b->blasBuildInfos)[ci.instanceID].clusterReferencesCount += 1;
      c.rb->numTotalTriangles += r.simple;
    }
    else
    {
      for(uint32_t tri = 0; tri < r.numTriangles; tri++)
      {
        uint32_t m = std::max(std::max(r.factors[tri][0], r.factors[tri][1]), r.factors[tri][2]);
        if(m > TC_TESSTABLE_SIZE)
          triOut.push_back({v, tri, (uint32_t)b->splitTriangleCounter++, true});
        else
          triOut.push_back({v, tri, b->partTriangleCounter++, false});
      }
    }
  }

  // phase 3: writes (parallel)
  const uint32_t sf = clampSplitFactor(k.splitFactor);
  parallelFor(nvis, numThreads, [&](size_t lo, size_t hi) {
    for(size_t v = lo; v < hi; v++)
    {
      if(alloc[v].vertexOffset == ~0u)
        continue;
      const tc_ClusterInfo&         ci = vis[v];
      const tc_RenderInstance&      in = c.inst[ci.instanceID];
      const tc_Cluster&             cl = P<const tc_Cluster>(in.clusters)[ci.clusterID];
      const tc_DisplacementTexture* tx = instanceTexture(a, in);
      f3*                           gv = P<f3>(b->genVertices);
      for(uint32_t vert = 0; vert < cl.numVertices; vert++)
      {
        uint32_t vi  = cl.firstLocalVertex + vert;
        f3       pos = ld3(in.positions, vi);
        if(tx)
        {
          const f2 uv = P<const f2>(in.texcoords)[vi];
          pos         = displace(pos, ld3(in.normals, vi), uv, tx, in, *c.view);
        }
        if(a->flags & TC_FLAG_RIPPLE)  // cluster_classify.comp.glsl:483-485
          pos = ripple(pos, ci.instanceID, in.geoHi.w, *c.view);
        gv[alloc[v].vertexOffset + vert] = pos;
      }
    }
  });
  parallelFor(triOut.size(), numThreads, [&](size_t lo, size_t hi) {
    for(size_t i = lo; i < hi; i++)
    {
      const TriOut& o = triOut[i];
      Rec&          r = recs[o.cluster];
      uint32_t      f[3] = {r.factors[o.tri][0], r.factors[o.tri][1], r.factors[o.tri][2]};
      tc_TessTriangleInfo info;
      info.cluster                       = vis[o.cluster];
      info.subTriangle.vtxEncoded[0]     = 0;
      info.subTriangle.vtxEncoded[1]     = TC_TESSTABLE_COORD_MAX;
      info.subTriangle.vtxEncoded[2]     = TC_TESSTABLE_COORD_MAX << 16;
      info.subTriangle.triangleID_config = o.tri;
      if(o.split)
      {
        if(o.offset >= k.maxSplitTriangles)
          continue;
        for(int j = 0; j < 3; j++)
          f[j] = splitFactor1(f[j], sf);
        uint32_t cfg = getConfig(f, info.subTriangle.vtxEncoded);
        info.subTriangle.triangleID_config |= cfg << 16;
        P<tc_TessTriangleInfo>(b->splitTriangles)[o.offset] = info;
      }
      else
      {
        if(o.offset >= k.maxPartTriangles)
          continue;
        uint32_t cfg = getConfig(f, info.subTriangle.vtxEncoded);
        info.subTriangle.triangleID_config |= cfg << 16;
        P<tc_TessTriangleInfo>(b->partTriangles)[o.offset] = info;
      }
    }
  });
}

// shaders/triangle_split.comp.glsl:146-331 + 598-632: one pass over
// [splitPassStart, splitPassEnd), children in (parent, child index) order
void tco_triangle_split_pass(const tco_table* t, const tc_frame_args* a, int numThreads)
{
  Ctx               c(a);
  tc_SceneBuilding* b     = c.b;
  const uint32_t    start = b->splitPassStart, end = b->splitPassEnd;
  const uint32_t    n     = end > start ? end - start : 0;
  const uint32_t    sf    = clampSplitFactor(a->caps.splitFactor);
  tc_TessTriangleInfo* items = P<tc_TessTriangleInfo>(b->splitTriangles);

  struct Child
  {
    tc_TessTriangleInfo info;
    bool                split;
  };
  std::vector<std::vector<Child>> children(n);

  parallelFor(n, numThreads, [&](size_t lo, size_t hi) {
    for(size_t i = lo; i < hi; i++)
    {
      const tc_TessTriangleInfo parent = items[start + i];
      const uint32_t            cfg    = parent.subTriangle.triangleID_config >> 16;
      const uint32_t            triID  = parent.subTriangle.triangleID_config & 0xFFFF;
      const tc_RenderInstance&  in     = c.inst[parent.cluster.instanceID];
      const tc_Cluster&         cl     = P<const tc_Cluster>(in.clusters)[parent.cluster.clusterID];
      const uint8_t*            lt     = P<const uint8_t>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      // triangle_split.comp.glsl:146-180 fillBaseVertices
      f3 bp[3], bb[3];
      for(int k = 0; k < 3; k++)
      {
        bp[k] = xform_point(in.worldMatrix.m, ld3(in.positions, cl.firstLocalVertex + lt[triID * 3 + k]));
        bb[k] = decodeBary(parent.subTriangle.vtxEncoded[k]);
      }
      const uint32_t nt = t->entries[cfgIndex(cfg)].numTriangles;
      children[i].resize(nt);
      for(uint32_t sub = 0; sub < nt; sub++)
      {
        // triangle_split.comp.glsl:201-331 processSubTask
        tc_TessTriangleInfo child = parent;
        uint32_t            tv[3];
        cfgTriangle(t, cfg, sub, tv);
        for(int v = 0; v < 3; v++)
        {
          f3 vb                          = cfgVertex(t, cfg, tv[v]);
          child.subTriangle.vtxEncoded[v] = encodeBary(interp3(bb, vb));
        }
        f3 wp[3];
        for(int v = 0; v < 3; v++)
          wp[v] = interp3(bp, decodeBary(child.subTriangle.vtxEncoded[v]));
        uint32_t f[3];
        tessFactors(wp[0], wp[1], wp[2], c.fp, f);
        uint32_t m     = std::max(std::max(f[0], f[1]), f[2]);
        bool     split = m > TC_TESSTABLE_SIZE;
        if(split)
          for(int j = 0; j < 3; j++)
            f[j] = splitFactor1(f[j], sf);
        uint32_t ncfg                     = getConfig(f, child.subTriangle.vtxEncoded);
        child.subTriangle.triangleID_config = (child.subTriangle.triangleID_config & 0xFFFFu) | (ncfg << 16);
        children[i][sub]                  = {child, split};
      }
    }
  });

  const bool trans = (a->flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X)) != 0;
  for(uint32_t i = 0; i < n; i++)
    for(const Child& ch : children[i])
    {
      if(ch.split)
      {
        uint32_t off = b->splitWriteCounter++;
        if(off < a->caps.maxSplitTriangles)
          items[off] = ch.info;
      }
      else if(trans)
      {
        // build.glsl:68-82 through the two-sided counter, one child at a time;
        // partTriangleCounter keeps the end of the written front
        // (triangle_split.comp.glsl:321-328)
        const uint32_t x = (uint32_t)b->dualPartTriangleCounter, y = (uint32_t)(b->dualPartTriangleCounter >> 32);
        b->dualPartTriangleCounter += 1;
        if((uint64_t)x + y + 2 <= a->caps.maxPartTriangles)
        {
          P<tc_TessTriangleInfo>(b->partTriangles)[x] = ch.info;
          b->partTriangleCounter                      = std::max(b->partTriangleCounter, x + 1);
        }
      }
      else
      {
        uint32_t off = b->partTriangleCounter++;
        if(off < a->caps.maxPartTriangles)
          P<tc_TessTriangleInfo>(b->partTriangles)[off] = ch.info;
      }
    }
}

// shaders/triangle_tess_template_instantiate.comp.glsl:126-373
void tco_triangle_instantiate(const tco_table* t, const tc_frame_args* a, int numThreads)
{
  Ctx                        c(a);
  tc_SceneBuilding*          b     = c.b;
  const uint32_t             nparts = b->partTriangleCounter;
  const tc_TessTriangleInfo* parts = P<const tc_TessTriangleInfo>(b->partTriangles);
  const tc_caps&             k     = a->caps;
  std::vector<uint32_t>      vertexOffsets(nparts, ~0u);

  for(uint32_t p = 0; p < nparts; p++)
  {
    const tc_TessTriangleInfo& info   = parts[p];
    const uint32_t             cfg    = info.subTriangle.triangleID_config >> 16;
    const tc_TessTableEntry&   e      = t->entries[cfgIndex(cfg)];
    uint32_t                   genOffset = b->genClusterCounter++;
    uint64_t                   dataSize  = t->templateInstantiationSizes[cfgIndex(cfg)];
    uint64_t                   dataOffset = b->genClusterDataCounter;
    b->genClusterDataCounter += dataSize;
    uint32_t vertexOffset = b->genVertexCounter;
    b->genVertexCounter += e.numVertices;
    if((uint64_t)vertexOffset + e.numVertices > k.maxGeneratedVertices || genOffset + 1 > k.maxGeneratedClusters
       || dataOffset + dataSize > c.maxDataBytes)
      continue;
    tc_TemplateInstantiateInfo ti;
    ti.clusterIdOffset        = p | (TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED << 30);
    ti.geometryIndexOffset    = 0;
    ti.clusterTemplateAddress = t->templateAddresses[cfgIndex(cfg)];
    ti.vertexBufferAddress    = b->genVertices + uint64_t(vertexOffset) * 12;
    ti.vertexBufferStride     = 12;
    uint32_t tempOffset       = b->tempInstantiateCounter++;
    P<tc_TemplateInstantiateInfo>(b->tempInstantiations)[tempOffset] = ti;
    P<uint32_t>(b->tempInstanceIDs)[tempOffset]                      = info.cluster.instanceID;
    P<uint64_t>(b->tempClusterAddresses)[tempOffset]                 = b->genClusterData + dataOffset;
    P<tc_BlasBuildInfo>(b->blasBuildInfos)[info.cluster.instanceID].clusterReferencesCount += 1;
    c.rb->numTotalTriangles += e.numTriangles;
    vertexOffsets[p] = vertexOffset;
  }

  parallelFor(nparts, numThreads, [&](size_t lo, size_t hi) {
    for(size_t p = lo; p < hi; p++)
    {
      if(vertexOffsets[p] == ~0u)
        continue;
      const tc_TessTriangleInfo&    info = parts[p];
      const uint32_t                cfg  = info.subTriangle.triangleID_config >> 16;
      const uint32_t                triID = info.subTriangle.triangleID_config & 0xFFFF;
      const tc_RenderInstance&      in   = c.inst[info.cluster.instanceID];
      const tc_Cluster&             cl   = P<const tc_Cluster>(in.clusters)[info.cluster.clusterID];
      const uint8_t*                lt   = P<const uint8_t>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      const tc_DisplacementTexture* tx   = instanceTexture(a, in);
      f3                            bb[3], bpos[3], bnrm[3];
      f2                            buv[3];
      for(int j = 0; j < 3; j++)
      {
        uint32_t vi = cl.firstLocalVertex + lt[triID * 3 + j];
        bb[j]       = decodeBary(info.subTriangle.vtxEncoded[j]);
        bpos[j]     = ld3(in.positions, vi);
        bnrm[j]     = normalize3(ld3(in.normals, vi));
        buv[j]      = P<const f2>(in.texcoords)[vi];
      }
      const uint32_t nv = t->entries[cfgIndex(cfg)].numVertices;
      f3*            gv = P<f3>(b->genVertices);
      // triangle_tess_template_instantiate.comp.glsl:333-370
      const bool pn = (a->flags & TC_FLAG_PN) != 0, rip = (a->flags & TC_FLAG_RIPPLE) != 0;
      BasePN     basePN;
      if(pn)
        basePN = setupPN(bpos, bnrm);
      for(uint32_t vert = 0; vert < nv; vert++)
      {
        f3 w   = interp3(bb, cfgVertex(t, cfg, vert));
        f3 pos = pn ? getPN(basePN, w) : interp3(bpos, w);
        if(tx)
          pos = displace(pos, interp3(bnrm, w), interp2(buv, w), tx, in, *c.view);
        if(rip)
          pos = ripple(pos, info.cluster.instanceID, in.geoHi.w, *c.view);
        gv[vertexOffsets[p] + vert] = pos;
      }
    }
  });
}

// shaders/blas_setup_insertion.comp.glsl:100-116 (instance order = exclusive scan)
void tco_blas_setup_insertion(const tc_frame_args* a)
{
  Ctx               c(a);
  tc_SceneBuilding* b = c.b;
  tc_BlasBuildInfo* infos = P<tc_BlasBuildInfo>(b->blasBuildInfos);
  for(uint32_t i = 0; i < b->numRenderInstances; i++)
  {
    uint32_t count  = infos[i].clusterReferencesCount;
    uint32_t offset = b->blasClusterCounter;
    b->blasClusterCounter += count;
    infos[i].clusterReferencesCount  = 0;
    infos[i].clusterReferencesStride = 8;
    infos[i].clusterReferences       = b->blasClusterAddresses + uint64_t(offset) * 8;
    if(b->blasBuildSizes)
      c.rb->numBlasActualSizes += P<const uint32_t>(b->blasBuildSizes)[i];
  }
}

// shaders/blas_clusters_insert.comp.glsl:97-136 (template instantiations in
// order, then transient builds in order)
void tco_blas_clusters_insert(const tc_frame_args* a)
{
  Ctx               c(a);
  tc_SceneBuilding* b     = c.b;
  tc_BlasBuildInfo* infos = P<tc_BlasBuildInfo>(b->blasBuildInfos);
  for(uint32_t j = 0; j < b->tempInstantiateCounter; j++)
  {
    uint32_t inst = P<const uint32_t>(b->tempInstanceIDs)[j];
    uint64_t addr = P<const uint64_t>(b->tempClusterAddresses)[j];
    uint32_t size = b->tempClusterSizes ? P<const uint32_t>(b->tempClusterSizes)[j] : 0;
    uint32_t idx  = infos[inst].clusterReferencesCount++;
    P<uint64_t>(infos[inst].clusterReferences)[idx] = addr;
    c.rb->numGenActualDatas += size;
  }
  // the second dispatch (push.instanceID 1): transient builds, after every
  // template instantiation of the frame
  if(a->flags & (TC_FLAG_TRANSIENT_1X | TC_FLAG_TRANSIENT_2X))
    for(uint32_t j = 0; j < b->transBuildCounter; j++)
    {
      uint32_t inst = P<const uint32_t>(b->transInstanceIDs)[j];
      uint64_t addr = P<const uint64_t>(b->transClusterAddresses)[j];
      uint32_t size = b->transClusterSizes ? P<const uint32_t>(b->transClusterSizes)[j] : 0;
      uint32_t idx  = infos[inst].clusterReferencesCount++;
      P<uint64_t>(infos[inst].clusterReferences)[idx] = addr;
      c.rb->numGenActualDatas += size;
    }
}

// src/renderer_raytrace_clusters_tess.cpp:410-692 (compute part)
// render_raytrace_clusters.rchit.glsl:131-214 (RT target; the transient-build
// modes when the frame's flags have them): a cluster-ray-tracing hit to the base triangle, its vertices and
// base barycentrics. The barycentric compositions are written out as separate
// multiplies and adds in the shader's left-to-right order.
void tco_decode_hits(const tco_table* t, const tc_frame_args* a, const tc_hit* hits, uint32_t count, tc_base_hit* out)
{
  Ctx                        c(a);
  const tc_SceneBuilding*    b     = c.b;
  const tc_TessTriangleInfo* parts = P<const tc_TessTriangleInfo>(b->partTriangles);
  const tc_FrameConstants*   view  = reinterpret_cast<const tc_FrameConstants*>(a->view);
  const bool                 visTriangles = view->visualize == TC_VISUALIZE_TRIANGLES;
  auto                       compose = [](f3 p, f3 q, f3 r, f3 w) {
    f3 o;
    o.x = (p.x * w.x + q.x * w.y) + r.x * w.z;
    o.y = (p.y * w.x + q.y * w.y) + r.y * w.z;
    o.z = (p.z * w.x + q.z * w.y) + r.z * w.z;
    return o;
  };
  for(uint32_t i = 0; i < count; i++)
  {
    const tc_hit& h    = hits[i];
    tc_base_hit   r    = {};
    uint32_t      mode = h.clusterID >> 30, clusterID = h.clusterID & 0x3FFFFFFFu;
    uint32_t      triangleID = h.triangleID, subTriangleID = h.triangleID, cfg = 0;
    uint32_t      partID     = visTriangles ? triangleID + 1 : 0u;
    uint32_t      enc[3]     = {0, 0, 0};
    bool          tess       = mode == TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED;
    r.status                 = TC_HIT_OK;
    if((mode == TC_RT_CLUSTER_MODE_1X_SUBSET_CLUSTER && !(a->flags & TC_FLAG_TRANSIENT_1X))
       || (mode == TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED && !(a->flags & TC_FLAG_TRANSIENT_2X)))
      r.status = TC_HIT_UNSUPPORTED_MODE;
    else if(h.instanceID >= a->numInstances)
      r.status = TC_HIT_OUT_OF_RANGE;
    else if(mode == TC_RT_CLUSTER_MODE_1X_SUBSET_CLUSTER || mode == TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED)
    {
      // rchit.glsl:150-180: the ClusterInfo header and the triangle map of a
      // transient build at the back of partTriangles
      const bool     mini = mode == TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED;
      const uint64_t need = mini ? 10ull + 2ull * triangleID : 9ull + triangleID;  // header + map entry, in bytes
      if(clusterID >= a->caps.maxPartTriangles || need > uint64_t(a->caps.maxPartTriangles - clusterID) * 24
         || triangleID >= (mini ? 32u : 64u))
        r.status = TC_HIT_OUT_OF_RANGE;
      else
      {
        const uint8_t*       rec = P<const uint8_t>(b->partTriangles) + uint64_t(clusterID) * 24;
        const tc_ClusterInfo hdr = *reinterpret_cast<const tc_ClusterInfo*>(rec);
        if(mini)
        {
          uint16_t packed;
          std::memcpy(&packed, rec + 8 + 2 * triangleID, 2);
          triangleID    = packed & 0xFF;
          subTriangleID = (packed >> 8) & 4;  // the shader's mask (rchit.glsl:161), kept as written
          enc[0]        = 0;
          enc[1]        = TC_TESSTABLE_COORD_MAX;
          enc[2]        = TC_TESSTABLE_COORD_MAX << 16;
          uint32_t f[3] = {1u + ((packed >> 12) & 1u), 1u + ((packed >> 13) & 1u), 1u + (uint32_t)(packed >> 14)};
          cfg           = getConfig(f, enc);
          tess          = true;
        }
        else
          triangleID = rec[8 + triangleID];
        clusterID = hdr.clusterID;
        if(hdr.instanceID != h.instanceID || (tess && subTriangleID >= t->entries[cfgIndex(cfg)].numTriangles))
          r.status = TC_HIT_OUT_OF_RANGE;
      }
    }
    else if(mode == TC_RT_CLUSTER_MODE_SINGLE_TESSELLATED)
    {
      if(clusterID >= std::min(b->partTriangleCounter, a->caps.maxPartTriangles))
        r.status = TC_HIT_OUT_OF_RANGE;
      else
      {
        const tc_TessTriangleInfo& pt = parts[clusterID];
        triangleID                    = pt.subTriangle.triangleID_config & 0xFFFF;
        cfg                           = pt.subTriangle.triangleID_config >> 16;
        clusterID                     = pt.cluster.clusterID;
        for(int v = 0; v < 3; v++)
          enc[v] = pt.subTriangle.vtxEncoded[v];
        if(pt.cluster.instanceID != h.instanceID || subTriangleID >= t->entries[cfgIndex(cfg)].numTriangles)
          r.status = TC_HIT_OUT_OF_RANGE;
      }
    }
    const tc_RenderInstance* in = r.status == TC_HIT_OK ? &c.inst[h.instanceID] : nullptr;
    if(in && clusterID >= in->numClusters)
      r.status = TC_HIT_OUT_OF_RANGE;
    tc_Cluster cl = {};
    if(r.status == TC_HIT_OK)
    {
      cl = P<const tc_Cluster>(in->clusters)[clusterID];
      if(triangleID >= cl.numTriangles)
        r.status = TC_HIT_OUT_OF_RANGE;
    }
    if(r.status != TC_HIT_OK)
    {
      out[i] = r;
      continue;
    }
    const uint8_t* lt = P<const uint8_t>(in->clusterLocalTriangles) + cl.firstLocalTriangle;
    for(int v = 0; v < 3; v++)
      r.vertexIndices[v] = lt[triangleID * 3 + v] + cl.firstLocalVertex;
    const f3 w    = {(1.0f - h.barycentrics[0]) - h.barycentrics[1], h.barycentrics[0], h.barycentrics[1]};
    f3       base = w;
    if(tess)
    {
      partID = 0;
      for(int v = 0; v < 3; v++)
        partID ^= (enc[v] >> 20) | ((enc[v] >> 4) & 0xFFF);
      uint32_t tri[3];
      cfgTriangle(t, cfg, subTriangleID, tri);
      const f3 sub = compose(cfgVertex(t, cfg, tri[0]), cfgVertex(t, cfg, tri[1]), cfgVertex(t, cfg, tri[2]), w);
      base         = compose(decodeBary(enc[0]), decodeBary(enc[1]), decodeBary(enc[2]), sub);
      partID       = visTriangles ? subTriangleID * 3 : partID;
      partID       = triangleID | ((partID | 1u) << 8);
    }
    r.clusterID       = clusterID;
    r.triangleID      = triangleID;
    r.barycentrics[0] = base.x;
    r.barycentrics[1] = base.y;
    r.barycentrics[2] = base.z;
    r.partID          = partID;
    out[i]            = r;
  }
}

// render_raster_clusters_batched.task.glsl:115-215: per group of 32 parts the
// linear fill into batches (a batch ends at the last part whose running
// vertex and triangle sums both stay within the limits), then
// render_raster_clusters_batched.mesh.glsl:141-435: every part's vertices
// (the instantiation's displaced position, then world and clip space) and its
// table triangles with the batch-local indices and primitive IDs.
void tco_raster_batches(const tco_table* t, const tc_frame_args* a, const tc_raster_outputs* out)
{
  Ctx                        c(a);
  const tc_SceneBuilding*    b      = c.b;
  const uint32_t             nparts = std::min(b->partTriangleCounter, a->caps.maxPartTriangles);
  const tc_TessTriangleInfo* parts  = P<const tc_TessTriangleInfo>(b->partTriangles);
  tc_raster_batch*           batches = P<tc_raster_batch>(out->batches);
  float*                     clip   = P<float>(out->clipPositions);
  float*                     world  = P<float>(out->worldPositions);
  uint8_t*                   idx    = P<uint8_t>(out->indices);
  uint32_t*                  prim   = P<uint32_t>(out->primitiveIDs);
  const bool                 visTriangles = c.view->visualize == TC_VISUALIZE_TRIANGLES;
  const bool                 pn = (a->flags & TC_FLAG_PN) != 0, rip = (a->flags & TC_FLAG_RIPPLE) != 0;
  uint32_t                   nb = 0, nv = 0, ntr = 0;
  for(uint32_t g0 = 0; g0 < nparts; g0 += 32)
  {
    const uint32_t local = std::min(32u, nparts - g0);
    uint32_t       sumV[32], sumT[32];
    uint32_t       accV = 0, accT = 0;
    for(uint32_t i = 0; i < 32; i++)
    {
      uint32_t v = TC_RASTER_BATCH_VERTICES, tr = TC_RASTER_BATCH_TRIANGLES;
      if(i < local)
      {
        const tc_TessTableEntry& e = t->entries[cfgIndex(parts[g0 + i].subTriangle.triangleID_config >> 16)];
        v = e.numVertices, tr = e.numTriangles;
      }
      accV += v, accT += tr;
      sumV[i] = accV, sumT[i] = accT;
    }
    uint32_t start = 0, lastV = 0, lastT = 0, left = local, batchIndex = 0;
    while(left != 0 && batchIndex < 32)
    {
      int end = -1;
      for(uint32_t i = 0; i < 32; i++)  // unsigned differences: parts before the batch do not fit
        if(sumV[i] - lastV <= TC_RASTER_BATCH_VERTICES && sumT[i] - lastT <= TC_RASTER_BATCH_TRIANGLES)
          end = (int)i;
      const uint32_t count = 1 + (uint32_t)end - start;
      if(nb < out->maxBatches)
      {
        tc_raster_batch& r = batches[nb];
        r.firstPart        = g0 + start;
        r.partCount        = std::min(count, left);
        r.firstVertex      = nv + (start ? sumV[start - 1] : 0);
        r.firstTriangle    = ntr + (start ? sumT[start - 1] : 0);
        r.numVertices      = sumV[end] - (start ? sumV[start - 1] : 0);
        r.numTriangles     = sumT[end] - (start ? sumT[start - 1] : 0);
      }
      nb++;
      lastV = sumV[end], lastT = sumT[end];
      start = (uint32_t)end + 1;
      left -= std::min(count, left);
      batchIndex++;
    }
    // the parts' vertices and triangles (group-local prefix sums, then the
    // running totals of the groups before)
    for(uint32_t i = 0; i < local; i++)
    {
      const tc_TessTriangleInfo& info  = parts[g0 + i];
      const uint32_t             cfg   = info.subTriangle.triangleID_config >> 16;
      const uint32_t             triID = info.subTriangle.triangleID_config & 0xFFFF;
      const tc_TessTableEntry&   e     = t->entries[cfgIndex(cfg)];
      const uint32_t             v0    = nv + sumV[i] - e.numVertices;
      const uint32_t             t0    = ntr + sumT[i] - e.numTriangles;
      // the batch-local first vertex of this part: vertices since its batch's first part
      uint32_t batchFirstV = 0;
      for(uint32_t q = 0, s0 = 0, lv = 0, lt = 0; q < 32 && s0 <= i; q++)
      {
        int end = -1;
        for(uint32_t j = 0; j < 32; j++)
          if(sumV[j] - lv <= TC_RASTER_BATCH_VERTICES && sumT[j] - lt <= TC_RASTER_BATCH_TRIANGLES)
            end = (int)j;
        if(i <= (uint32_t)end)
        {
          batchFirstV = s0 ? sumV[s0 - 1] : 0;
          break;
        }
        lv = sumV[end], lt = sumT[end], s0 = (uint32_t)end + 1;
      }
      const tc_RenderInstance&      in = c.inst[info.cluster.instanceID];
      const tc_Cluster&             cl = P<const tc_Cluster>(in.clusters)[info.cluster.clusterID];
      const uint8_t*                lt = P<const uint8_t>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      const tc_DisplacementTexture* tx = instanceTexture(a, in);
      f3                            bb[3], bpos[3], bnrm[3];
      f2                            buv[3];
      uint32_t                      partID = 0;
      for(int j = 0; j < 3; j++)
      {
        uint32_t vi = cl.firstLocalVertex + lt[triID * 3 + j];
        bb[j]       = decodeBary(info.subTriangle.vtxEncoded[j]);
        bpos[j]     = ld3(in.positions, vi);
        bnrm[j]     = normalize3(ld3(in.normals, vi));
        buv[j]      = P<const f2>(in.texcoords)[vi];
        partID ^= (info.subTriangle.vtxEncoded[j] >> 20) | ((info.subTriangle.vtxEncoded[j] >> 4) & 0xFFF);
      }
      BasePN basePN;
      if(pn)
        basePN = setupPN(bpos, bnrm);
      const float* vp = c.view->viewProjMatrix.m;
      for(uint32_t vert = 0; vert < e.numVertices; vert++)
      {
        if(v0 + vert >= out->maxVertices)
          break;
        f3 w   = interp3(bb, cfgVertex(t, cfg, vert));
        f3 pos = pn ? getPN(basePN, w) : interp3(bpos, w);
        if(tx)
          pos = displace(pos, interp3(bnrm, w), interp2(buv, w), tx, in, *c.view);
        if(rip)
          pos = ripple(pos, info.cluster.instanceID, in.geoHi.w, *c.view);
        const f3 wp = xform_point(in.worldMatrix.m, pos);
        const f3 cp = xform_point(vp, wp);
        float*   wo = world + 3 * uint64_t(v0 + vert);
        float*   co = clip + 4 * uint64_t(v0 + vert);
        wo[0] = wp.x, wo[1] = wp.y, wo[2] = wp.z;
        co[0] = cp.x, co[1] = cp.y, co[2] = cp.z;
        co[3] = ((vp[3] * wp.x + vp[7] * wp.y) + vp[11] * wp.z) + vp[15];
      }
      for(uint32_t tri = 0; tri < e.numTriangles; tri++)
      {
        if(t0 + tri >= out->maxTriangles)
          break;
        uint32_t ct[3];
        cfgTriangle(t, cfg, tri, ct);
        const uint32_t vs = v0 - nv - batchFirstV;  // the part's first vertex within its batch
        for(int j = 0; j < 3; j++)
          idx[3 * uint64_t(t0 + tri) + j] = (uint8_t)(ct[j] + vs);
        const uint32_t pid   = visTriangles ? tri * 3 : partID;
        prim[t0 + tri]       = (triID & 0xFF) | ((pid | 1u) << 8);
      }
    }
    nv += sumV[local - 1], ntr += sumT[local - 1];
  }
  uint32_t* counts = P<uint32_t>(out->counts);
  counts[0] = nb, counts[1] = nv, counts[2] = ntr;
}

int tco_frame_build(const tco_table* t, const tc_frame_args* a, int numThreads, uint32_t* partRunStarts)
{
  tc_SceneBuilding* b = P<tc_SceneBuilding>(a->build);
  tco_frame_begin(a);
  tco_instances_classify(a);
  tco_clusters_cull(a);
  tco_build_setup(a, TC_BUILD_SETUP_CLASSIFY);
  tco_cluster_classify(t, a, numThreads);
  tco_build_setup(a, TC_BUILD_SETUP_SPLIT);
  uint32_t passes = tco_split_pass_count(a->caps.splitFactor);
  if(partRunStarts)
  {
    partRunStarts[0] = 0;
    partRunStarts[1] = b->partTriangleCounter;
  }
  for(uint32_t p = 0; p < passes; p++)
  {
    tco_triangle_split_pass(t, a, numThreads);
    if(partRunStarts)
      partRunStarts[p + 2] = b->partTriangleCounter;
    if(p + 1 < passes)
      tco_build_setup(a, TC_BUILD_SETUP_SPLIT_PASS);
  }
  tco_build_setup(a, TC_BUILD_SETUP_INSTANTIATE_TESS);
  tco_triangle_instantiate(t, a, numThreads);
  tco_build_setup(a, TC_BUILD_SETUP_BUILD_BLAS);
  tco_blas_setup_insertion(a);
  tco_blas_clusters_insert(a);
  return 0;
}

}  // extern "C"

namespace {

constexpr uint32_t kClusterInfoBytes = 8, kTessInfoBytes = 24;
constexpr uint32_t kMiniBatchTris    = TC_2X_MINI_BATCHSIZE * TC_2X_MINI_TRIANGLES;
constexpr uint32_t kMiniBatchVerts   = TC_2X_MINI_BATCHSIZE * TC_2X_MINI_VERTICES;

// build.glsl:52-82: the two-sided part counter. The low half counts part
// triangles from the front of partTriangles, the high half the slots taken
// from its back by transient builds; an allocation that would make them meet
// gets the out-of-range offset maxPartTriangles (the counter still advances).
struct DualCounter
{
  uint64_t& v;
  uint32_t  max;
  uint32_t front(uint32_t n)
  {
    const uint32_t x = (uint32_t)v, y = (uint32_t)(v >> 32);
    v += n;
    return (uint64_t)x + y + n + 1 > max ? max : x;
  }
  uint32_t back(uint32_t m)
  {
    const uint32_t x = (uint32_t)v, y = (uint32_t)(v >> 32);
    v += (uint64_t)m << 32;
    return (uint64_t)x + y + m + 1 > max ? max : max - y - m;
  }
};

// cluster_classify.comp.glsl:401-431 / 751-786
tc_ClasBuildInfo clasBuildInfo(uint32_t mode, uint32_t partOffset, uint32_t numTriangles, uint32_t numVertices,
                               uint32_t truncateBits, uint64_t vertexBuffer)
{
  tc_ClasBuildInfo bi                  = {};
  bi.clusterID                         = (mode << 30) | partOffset;
  bi.clusterFlags                      = 0;
  bi.packed                            = numTriangles | (numVertices << 9) | (truncateBits << 18) | (1u << 24);
  bi.baseGeometryIndexAndFlags         = 4u << 29;
  bi.indexBufferStride                 = 1;
  bi.vertexBufferStride                = 12;
  bi.geometryIndexAndFlagsBufferStride = 0;
  bi.opacityMicromapIndexBufferStride  = 0;
  bi.vertexBuffer                      = vertexBuffer;
  bi.indexBuffer                       = vertexBuffer + uint64_t(numVertices) * 12;
  return bi;
}

inline uint32_t maxFactor(const uint32_t f[3]) { return std::max(std::max(f[0], f[1]), f[2]); }

// cluster_classify.comp.glsl:254-905 with TESS_USE_1X_TRANSIENTBUILDS and / or
// TESS_USE_2X_TRANSIENTBUILDS, in the canonical order: clusters in visible
// order; within a cluster the full-cluster / 1X allocation, then per 32-triangle
// chunk (the reference's subgroup) its part and split allocations followed by
// its 2X batches in triangle order. The bytes the reference leaves unwritten
// inside an allocation (index and map padding, unused batch vertex slots) are
// written as zeros.
void classifyTransient(const tco_table* t, const tc_frame_args* a, std::vector<ClassifyRec>& recs, int numThreads)
{
  Ctx                   c(a);
  tc_SceneBuilding*     b    = c.b;
  const tc_caps&        k    = a->caps;
  const uint32_t        nvis = b->visibleClusterCounter;
  const tc_ClusterInfo* vis  = P<const tc_ClusterInfo>(b->visibleClusters);
  const bool            t1   = (a->flags & TC_FLAG_TRANSIENT_1X) != 0;
  const bool            t2   = (a->flags & TC_FLAG_TRANSIENT_2X) != 0;
  const uint32_t*       basic = P<const uint32_t>(b->basicClusterSizes);
  DualCounter           dual{b->dualPartTriangleCounter, k.maxPartTriangles};
  tc_BlasBuildInfo*     blas = P<tc_BlasBuildInfo>(b->blasBuildInfos);

  // vertex jobs: full clusters and 1X subsets (the cluster's vertices), 2X batches
  struct ClusterJob
  {
    uint32_t v, vertexOffset, partOffset, partSlots;  // partSlots 0: full cluster
  };
  struct MiniJob
  {
    uint32_t v, vertexOffset, partOffset, count;
    uint32_t tris[TC_2X_MINI_BATCHSIZE];
  };
  struct TriOut
  {
    uint32_t cluster, tri, offset;
    bool     split;
  };
  std::vector<ClusterJob> clusterJobs;
  std::vector<MiniJob>    miniJobs;
  std::vector<TriOut>     triOut;
  auto accepts = [&](uint64_t vertexOffset, uint32_t vertexSize, uint32_t genOffset, uint64_t dataOffset,
                     uint64_t dataSize, uint64_t partOffset, uint32_t partSize) {
    return !((vertexOffset + vertexSize > k.maxGeneratedVertices) || (genOffset + 1ull > k.maxGeneratedClusters)
             || (dataOffset + dataSize > c.maxDataBytes) || (partOffset + partSize > k.maxPartTriangles));
  };

  for(uint32_t v = 0; v < nvis; v++)
  {
    const tc_ClusterInfo&    ci     = vis[v];
    const tc_RenderInstance& in     = c.inst[ci.instanceID];
    const tc_Cluster&        cl     = P<const tc_Cluster>(in.clusters)[ci.clusterID];
    const ClassifyRec&       r      = recs[v];
    const uint32_t           nt     = r.numTriangles, simple = r.simple, nv = cl.numVertices;
    const bool               isFull = simple == nt;
    const bool               oneX   = t1 && !isFull && simple > 1;
    // :254-437 full cluster or 1X subset
    if(isFull || oneX)
    {
      if(isFull)
        c.rb->numFullClusters += 1;
      const uint32_t genOffset  = b->genClusterCounter++;
      const uint64_t dataSize   = isFull ? P<const uint32_t>(in.clusterTemplateInstantiatonSizes)[ci.clusterID] : basic[simple];
      const uint32_t vertexSize = nv + (isFull ? 0u : (simple * 3 + 11) / 12);
      const uint32_t partSize   = isFull ? 0u : (kClusterInfoBytes + simple + kTessInfoBytes - 1) / kTessInfoBytes;
      const uint32_t partOffset = isFull ? 0u : dual.back(partSize);
      const uint64_t dataOffset = b->genClusterDataCounter;
      b->genClusterDataCounter += dataSize;
      const uint32_t vertexOffset = b->genVertexCounter;
      b->genVertexCounter += vertexSize;
      if(accepts(vertexOffset, vertexSize, genOffset, dataOffset, dataSize, partOffset, partSize))
      {
        if(isFull)
        {
          const uint32_t             tempOffset = b->tempInstantiateCounter++;
          tc_TemplateInstantiateInfo ti;
          ti.clusterIdOffset        = 0;
          ti.geometryIndexOffset    = 0;
          ti.clusterTemplateAddress = P<const uint64_t>(in.clusterTemplateAdresses)[ci.clusterID];
          ti.vertexBufferAddress    = b->genVertices + uint64_t(vertexOffset) * 12;
          ti.vertexBufferStride     = 12;
          P<tc_TemplateInstantiateInfo>(b->tempInstantiations)[tempOffset] = ti;
          P<uint32_t>(b->tempInstanceIDs)[tempOffset]                      = ci.instanceID;
          P<uint64_t>(b->tempClusterAddresses)[tempOffset]                 = b->genClusterData + dataOffset;
          if((a->flags & TC_FLAG_WRITE_FULLCLUSTERS) && b->fullClusters)
            P<tc_ClusterInfo>(b->fullClusters)[tempOffset] = ci;
        }
        else
        {
          const uint32_t transOffset = b->transBuildCounter++;
          P<tc_ClasBuildInfo>(b->transBuilds)[transOffset] =
              clasBuildInfo(TC_RT_CLUSTER_MODE_1X_SUBSET_CLUSTER, partOffset, simple, nv, b->positionTruncateBitCount,
                            b->genVertices + uint64_t(vertexOffset) * 12);
          P<uint32_t>(b->transInstanceIDs)[transOffset]      = ci.instanceID;
          P<uint64_t>(b->transClusterAddresses)[transOffset] = b->genClusterData + dataOffset;
        }
        clusterJobs.push_back({v, vertexOffset, partOffset, partSize});
        blas[ci.instanceID].clusterReferencesCount += 1;
        c.rb->numTotalTriangles += simple;
      }
    }
    if(isFull)
      continue;
    // :543-905 the remaining triangles, one 32-triangle chunk at a time
    for(uint32_t t0 = 0; t0 < nt; t0 += 32)
    {
      const uint32_t t1e = std::min(nt, t0 + 32);
      uint32_t       nPart = 0, nSplit = 0;
      uint32_t       mini[32], nMini = 0;
      uint8_t        kind[32];  // 0 handled by the 1X subset, 1 split, 2 part, 3 mini
      for(uint32_t tri = t0; tri < t1e; tri++)
      {
        const uint32_t m = maxFactor(r.factors[tri]);
        uint8_t        kd;
        if(oneX && m == 1)
          kd = 0;
        else if(m > TC_TESSTABLE_SIZE)
          kd = 1;
        else if(t2 && m <= 2)
          kd = 3;
        else
          kd = 2;
        kind[tri - t0] = kd;
        nSplit += kd == 1;
        nPart += kd == 2;
        if(kd == 3)
          mini[nMini++] = tri;
      }
      const uint32_t splitBase = (uint32_t)b->splitTriangleCounter;
      b->splitTriangleCounter += (int32_t)nSplit;
      const uint32_t partBase = dual.front(nPart);
      if(nPart && partBase < k.maxPartTriangles)  // written: the front's written end
        b->partTriangleCounter = std::max(b->partTriangleCounter, partBase + nPart);
      uint32_t is = 0, ip = 0;
      for(uint32_t tri = t0; tri < t1e; tri++)
      {
        if(kind[tri - t0] == 1)
          triOut.push_back({v, tri, splitBase + is++, true});
        else if(kind[tri - t0] == 2)
          triOut.push_back({v, tri, partBase + ip++, false});
      }
      // :675-790 the chunk's 2X batches
      for(uint32_t m0 = 0; m0 < nMini; m0 += TC_2X_MINI_BATCHSIZE)
      {
        MiniJob job = {};
        job.v       = v;
        job.count   = std::min(TC_2X_MINI_BATCHSIZE, nMini - m0);
        uint32_t numBatchTris = 0;
        for(uint32_t j = 0; j < job.count; j++)
        {
          job.tris[j]     = mini[m0 + j];
          uint32_t f[3]   = {r.factors[job.tris[j]][0], r.factors[job.tris[j]][1], r.factors[job.tris[j]][2]};
          uint32_t tv[3]  = {0, TC_TESSTABLE_COORD_MAX, TC_TESSTABLE_COORD_MAX << 16};
          numBatchTris += t->entries[cfgIndex(getConfig(f, tv))].numTriangles;
        }
        const uint64_t dataSize   = basic[kMiniBatchTris];
        const uint32_t vertexSize = kMiniBatchVerts + (kMiniBatchTris * 3 + 11) / 12;
        const uint32_t partSize   = (kClusterInfoBytes + kMiniBatchTris * 2 + kTessInfoBytes - 1) / kTessInfoBytes;
        const uint32_t genOffset  = b->genClusterCounter++;
        const uint32_t partOffset = dual.back(partSize);
        const uint64_t dataOffset = b->genClusterDataCounter;
        b->genClusterDataCounter += dataSize;
        const uint32_t vertexOffset = b->genVertexCounter;
        b->genVertexCounter += vertexSize;
        if(!accepts(vertexOffset, vertexSize, genOffset, dataOffset, dataSize, partOffset, partSize))
          continue;
        const uint32_t transOffset = b->transBuildCounter++;
        P<tc_ClasBuildInfo>(b->transBuilds)[transOffset] =
            clasBuildInfo(TC_RT_CLUSTER_MODE_2X_BATCHED_TESSELLATED, partOffset, numBatchTris, kMiniBatchVerts,
                          b->positionTruncateBitCount, b->genVertices + uint64_t(vertexOffset) * 12);
        P<uint32_t>(b->transInstanceIDs)[transOffset]      = ci.instanceID;
        P<uint64_t>(b->transClusterAddresses)[transOffset] = b->genClusterData + dataOffset;
        blas[ci.instanceID].clusterReferencesCount += 1;
        c.rb->numTotalTriangles += numBatchTris;
        job.vertexOffset = vertexOffset;
        job.partOffset   = partOffset;
        miniJobs.push_back(job);
      }
    }
  }

  uint8_t* gvb = P<uint8_t>(b->genVertices);
  uint8_t* ptb = P<uint8_t>(b->partTriangles);
  f3*      gv  = P<f3>(b->genVertices);
  const bool pn = (a->flags & TC_FLAG_PN) != 0, rip = (a->flags & TC_FLAG_RIPPLE) != 0;

  // full clusters and 1X subsets: the cluster's displaced vertices (:457-487),
  // then for a subset its indices after the vertices and its triangle map
  // after the ClusterInfo header (:489-535)
  parallelFor(clusterJobs.size(), numThreads, [&](size_t lo, size_t hi) {
    for(size_t j = lo; j < hi; j++)
    {
      const ClusterJob&             job = clusterJobs[j];
      const tc_ClusterInfo&         ci  = vis[job.v];
      const tc_RenderInstance&      in  = c.inst[ci.instanceID];
      const tc_Cluster&             cl  = P<const tc_Cluster>(in.clusters)[ci.clusterID];
      const tc_DisplacementTexture* tx  = instanceTexture(a, in);
      for(uint32_t vert = 0; vert < cl.numVertices; vert++)
      {
        uint32_t vi  = cl.firstLocalVertex + vert;
        f3       pos = ld3(in.positions, vi);
        if(tx)
          pos = displace(pos, ld3(in.normals, vi), P<const f2>(in.texcoords)[vi], tx, in, *c.view);
        if(rip)
          pos = ripple(pos, ci.instanceID, in.geoHi.w, *c.view);
        gv[job.vertexOffset + vert] = pos;
      }
      if(job.partSlots == 0)
        continue;
      const ClassifyRec& r      = recs[job.v];
      const uint8_t*     lt     = P<const uint8_t>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      uint8_t*           idx    = gvb + (uint64_t(job.vertexOffset) + cl.numVertices) * 12;
      uint8_t*           map    = ptb + uint64_t(job.partOffset) * kTessInfoBytes;
      std::memset(idx, 0, (size_t)((r.simple * 3 + 11) / 12) * 12);
      std::memset(map, 0, (size_t)job.partSlots * kTessInfoBytes);
      std::memcpy(map, &ci, kClusterInfoBytes);
      uint32_t out = 0;
      for(uint32_t tri = 0; tri < r.numTriangles; tri++)
        if(maxFactor(r.factors[tri]) == 1)
        {
          map[kClusterInfoBytes + out] = (uint8_t)tri;
          for(int q = 0; q < 3; q++)
            idx[out * 3 + q] = lt[tri * 3 + q];
          out++;
        }
    }
  });

  // 2X batches (:792-904): per base triangle its 3 to 6 vertices at its batch
  // slot, its table triangles' u16 map entries and u8 indices
  parallelFor(miniJobs.size(), numThreads, [&](size_t lo, size_t hi) {
    for(size_t j = lo; j < hi; j++)
    {
      const MiniJob&                job = miniJobs[j];
      const tc_ClusterInfo&         ci  = vis[job.v];
      const tc_RenderInstance&      in  = c.inst[ci.instanceID];
      const tc_Cluster&             cl  = P<const tc_Cluster>(in.clusters)[ci.clusterID];
      const uint8_t*                lt  = P<const uint8_t>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      const tc_DisplacementTexture* tx  = instanceTexture(a, in);
      const ClassifyRec&            r   = recs[job.v];
      uint8_t*                      idx = gvb + (uint64_t(job.vertexOffset) + kMiniBatchVerts) * 12;
      uint8_t*                      map = ptb + uint64_t(job.partOffset) * kTessInfoBytes;
      std::memset(gvb + uint64_t(job.vertexOffset) * 12, 0,
                  (size_t)(kMiniBatchVerts + (kMiniBatchTris * 3 + 11) / 12) * 12);
      std::memset(map, 0, (size_t)((kClusterInfoBytes + kMiniBatchTris * 2 + kTessInfoBytes - 1) / kTessInfoBytes) * kTessInfoBytes);
      std::memcpy(map, &ci, kClusterInfoBytes);
      uint32_t baseTris = 0;
      for(uint32_t rel = 0; rel < job.count; rel++)
      {
        const uint32_t tri  = job.tris[rel];
        uint32_t       f[3] = {r.factors[tri][0], r.factors[tri][1], r.factors[tri][2]};
        uint32_t       tv[3] = {0, TC_TESSTABLE_COORD_MAX, TC_TESSTABLE_COORD_MAX << 16};
        const uint32_t cfg   = getConfig(f, tv);
        const tc_TessTableEntry& e = t->entries[cfgIndex(cfg)];
        f3 bb[3], bpos[3], bnrm[3];
        f2 buv[3];
        for(int q = 0; q < 3; q++)
        {
          uint32_t vi = cl.firstLocalVertex + lt[tri * 3 + q];
          bb[q]       = decodeBary(tv[q]);
          bpos[q]     = ld3(in.positions, vi);
          bnrm[q]     = normalize3(ld3(in.normals, vi));
          buv[q]      = P<const f2>(in.texcoords)[vi];
        }
        BasePN basePN;
        if(pn)
          basePN = setupPN(bpos, bnrm);
        for(uint32_t vert = 0; vert < e.numVertices; vert++)
        {
          f3 w   = interp3(bb, cfgVertex(t, cfg, vert));
          f3 pos = pn ? getPN(basePN, w) : interp3(bpos, w);
          if(tx)
            pos = displace(pos, interp3(bnrm, w), interp2(buv, w), tx, in, *c.view);
          if(rip)
            pos = ripple(pos, ci.instanceID, in.geoHi.w, *c.view);
          gv[job.vertexOffset + rel * TC_2X_MINI_VERTICES + vert] = pos;
        }
        // the edge factors as computed (tess_getConfig takes them by value)
        const uint32_t* f0            = r.factors[tri];
        const uint32_t  packedFactors = (f0[0] - 1) | ((f0[1] - 1) << 1) | ((f0[2] - 1) << 2);
        for(uint32_t i = 0; i < e.numTriangles; i++)
        {
          const uint32_t triOffset = baseTris + i;
          const uint16_t m16       = (uint16_t)(tri | (i << 8) | (packedFactors << 12));
          std::memcpy(map + kClusterInfoBytes + 2 * triOffset, &m16, 2);
          uint32_t ct[3];
          cfgTriangle(t, cfg, i, ct);
          for(int q = 0; q < 3; q++)
            idx[triOffset * 3 + q] = (uint8_t)(ct[q] + rel * TC_2X_MINI_VERTICES);
        }
        baseTris += e.numTriangles;
      }
    }
  });

  // part and split triangles (:608-666)
  const uint32_t sf = clampSplitFactor(k.splitFactor);
  parallelFor(triOut.size(), numThreads, [&](size_t lo, size_t hi) {
    for(size_t i = lo; i < hi; i++)
    {
      const TriOut& o    = triOut[i];
      ClassifyRec&  r    = recs[o.cluster];
      uint32_t      f[3] = {r.factors[o.tri][0], r.factors[o.tri][1], r.factors[o.tri][2]};
      tc_TessTriangleInfo info;
      info.cluster                       = vis[o.cluster];
      info.subTriangle.vtxEncoded[0]     = 0;
      info.subTriangle.vtxEncoded[1]     = TC_TESSTABLE_COORD_MAX;
      info.subTriangle.vtxEncoded[2]     = TC_TESSTABLE_COORD_MAX << 16;
      info.subTriangle.triangleID_config = o.tri;
      if(o.split)
      {
        if(o.offset >= k.maxSplitTriangles)
          continue;
        for(int j = 0; j < 3; j++)
          f[j] = splitFactor1(f[j], sf);
        info.subTriangle.triangleID_config |= getConfig(f, info.subTriangle.vtxEncoded) << 16;
        P<tc_TessTriangleInfo>(b->splitTriangles)[o.offset] = info;
      }
      else
      {
        if(o.offset >= k.maxPartTriangles)
          continue;
        info.subTriangle.triangleID_config |= getConfig(f, info.subTriangle.vtxEncoded) << 16;
        P<tc_TessTriangleInfo>(b->partTriangles)[o.offset] = info;
      }
    }
  });
}

}  // namespace

// ===========================================================================
// FP64 twin and adjoint of the vertex generation
// ===========================================================================

namespace {

struct d3
{
  double x, y, z;
};
inline d3     operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3     operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3     operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dotd(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double lend(d3 a) { return std::sqrt(dotd(a, a)); }

struct ParamSource
{
  // nullptr entries -> use the float inputs of the instance / texture
  const double* const* positions = nullptr;
  const double* const* normals   = nullptr;
  const double* const* texels    = nullptr;

  d3 pos(const tc_RenderInstance& in, uint32_t inst, uint32_t vi) const
  {
    if(positions && positions[inst])
      return {positions[inst][3 * vi], positions[inst][3 * vi + 1], positions[inst][3 * vi + 2]};
    f3 p = ld3(in.positions, vi);
    return {p.x, p.y, p.z};
  }
  d3 nrm(const tc_RenderInstance& in, uint32_t inst, uint32_t vi) const
  {
    if(normals && normals[inst])
      return {normals[inst][3 * vi], normals[inst][3 * vi + 1], normals[inst][3 * vi + 2]};
    f3 p = ld3(in.normals, vi);
    return {p.x, p.y, p.z};
  }
  double tex(const tc_DisplacementTexture& tx, int texIndex, int x, int y) const
  {
    if(texels && texels[texIndex])
      return texels[texIndex][(size_t)y * tx.width + x];
    return texel(tx, x, y);
  }
};

struct TapsD
{
  int    x0, x1, y0, y1;
  double w00, w10, w01, w11;
};

TapsD tapsD(const tc_DisplacementTexture& tx, double u, double v)
{
  double x  = u * tx.width - 0.5;
  double y  = v * tx.height - 0.5;
  double xf = std::floor(x), yf = std::floor(y);
  double fx = x - xf, fy = y - yf;
  int    ix = (int)xf, iy = (int)yf;
  TapsD  t;
  t.x0  = wrapi(ix, (int)tx.width);
  t.x1  = wrapi(ix + 1, (int)tx.width);
  t.y0  = wrapi(iy, (int)tx.height);
  t.y1  = wrapi(iy + 1, (int)tx.height);
  t.w00 = (1 - fx) * (1 - fy);
  t.w10 = fx * (1 - fy);
  t.w01 = (1 - fx) * fy;
  t.w11 = fx * fy;
  return t;
}

// One generated vertex as a function of (up to) 3 base vertices with weights.
struct VertexJob
{
  uint32_t inst;
  uint32_t genIndex;
  int      nBase;  // 1 for full-cluster vertices, 3 for part vertices
  uint32_t vi[3];
  double   w[3];
};

template <class F>
void forEachGeneratedVertex(const tco_table* t, const tc_frame_args* a, F&& fn)
{
  const tc_SceneBuilding*          b     = P<const tc_SceneBuilding>(a->build);
  const tc_RenderInstance*         insts = P<const tc_RenderInstance>(a->instances);
  const tc_TemplateInstantiateInfo* ti   = P<const tc_TemplateInstantiateInfo>(b->tempInstantiations);
  const tc_TessTriangleInfo*       parts = P<const tc_TessTriangleInfo>(b->partTriangles);
  const tc_ClusterInfo*            fulls = P<const tc_ClusterInfo>(b->fullClusters);
  for(uint32_t j = 0; j < b->tempInstantiateCounter; j++)
  {
    uint32_t mode = ti[j].clusterIdOffset >> 30;
    uint32_t base = (uint32_t)((ti[j].vertexBufferAddress - b->genVertices) / 12);
    if(mode == TC_RT_CLUSTER_MODE_FULL_CLUSTER)
    {
      if(!fulls)
        continue;
      tc_ClusterInfo           ci = fulls[j];
      const tc_RenderInstance& in = insts[ci.instanceID];
      const tc_Cluster&        cl = P<const tc_Cluster>(in.clusters)[ci.clusterID];
      for(uint32_t v = 0; v < cl.numVertices; v++)
      {
        VertexJob job{ci.instanceID, base + v, 1, {cl.firstLocalVertex + v, 0, 0}, {1.0, 0, 0}};
        fn(job);
      }
    }
    else
    {
      const tc_TessTriangleInfo& info  = parts[ti[j].clusterIdOffset & 0x3FFFFFFFu];
      const uint32_t             cfg   = info.subTriangle.triangleID_config >> 16;
      const uint32_t             triID = info.subTriangle.triangleID_config & 0xFFFF;
      const tc_RenderInstance&   in    = insts[info.cluster.instanceID];
      const tc_Cluster&          cl    = P<const tc_Cluster>(in.clusters)[info.cluster.clusterID];
      const uint8_t*             lt    = P<const uint8_t>(in.clusterLocalTriangles) + cl.firstLocalTriangle;
      f3                         bb[3];
      for(int k = 0; k < 3; k++)
        bb[k] = decodeBary(info.subTriangle.vtxEncoded[k]);
      uint32_t nv = t->entries[cfgIndex(cfg)].numVertices;
      for(uint32_t v = 0; v < nv; v++)
      {
        f3 vb = cfgVertex(t, cfg, v);
        // exact in double: products of multiples of 2^-15
        double w0 = double(bb[0].x) * vb.x + double(bb[1].x) * vb.y + double(bb[2].x) * vb.z;
        double w1 = double(bb[0].y) * vb.x + double(bb[1].y) * vb.y + double(bb[2].y) * vb.z;
        double w2 = double(bb[0].z) * vb.x + double(bb[1].z) * vb.y + double(bb[2].z) * vb.z;
        VertexJob job{info.cluster.instanceID, base + v, 3,
                      {cl.firstLocalVertex + lt[triID * 3 + 0], cl.firstLocalVertex + lt[triID * 3 + 1],
                       cl.firstLocalVertex + lt[triID * 3 + 2]},
                      {w0, w1, w2}};
        fn(job);
      }
    }
  }
}

struct EvalOut
{
  d3     v;
  bool   displaced;
  d3     nhat[3];
  double nlen[3];
  d3     N;
  double Nlen;
  double h;
  double s;
  TapsD  taps;
  int    texIndex;
};

EvalOut evalVertexD(const tc_frame_args* a, const VertexJob& job, const ParamSource& src)
{
  const tc_RenderInstance& in = P<const tc_RenderInstance>(a->instances)[job.inst];
  const tc_FrameConstants& view = *P<const tc_FrameConstants>(a->view);
  EvalOut                  o{};
  d3                       pos = {0, 0, 0};
  for(int k = 0; k < job.nBase; k++)
    pos = pos + src.pos(in, job.inst, job.vi[k]) * job.w[k];
  o.v         = pos;
  const tc_DisplacementTexture* tx = instanceTexture(a, in);
  if(!tx)
    return o;
  o.displaced = true;
  o.texIndex  = in.displacementIndex;
  d3     N    = {0, 0, 0};
  double u = 0, v = 0;
  for(int k = 0; k < job.nBase; k++)
  {
    d3 n       = src.nrm(in, job.inst, job.vi[k]);
    o.nlen[k]  = lend(n);
    // full-cluster vertices normalise once (cluster_classify.comp.glsl:474-477),
    // part vertices normalise at load and after interpolation (instantiate :329,:363)
    o.nhat[k]  = job.nBase == 3 ? n * (1.0 / o.nlen[k]) : n;
    N          = N + o.nhat[k] * job.w[k];
    f2 uv      = P<const f2>(in.texcoords)[job.vi[k]];
    u += job.w[k] * uv.x;
    v += job.w[k] * uv.y;
  }
  o.N    = N;
  o.Nlen = lend(N);
  d3 m   = N * (1.0 / o.Nlen);
  o.taps = tapsD(*tx, u, v);
  double B = o.taps.w00 * src.tex(*tx, o.texIndex, o.taps.x0, o.taps.y0) + o.taps.w10 * src.tex(*tx, o.texIndex, o.taps.x1, o.taps.y0)
             + o.taps.w01 * src.tex(*tx, o.texIndex, o.taps.x0, o.taps.y1) + o.taps.w11 * src.tex(*tx, o.texIndex, o.taps.x1, o.taps.y1);
  o.s  = double(in.displacementScale) * double(view.displacementScale);
  o.h  = B * o.s + double(in.displacementOffset) + double(view.displacementOffset);
  o.v  = pos + m * o.h;
  return o;
}

}  // namespace

extern "C" {

uint64_t tco_generate_vertices_f64(const tco_table* t, const tc_frame_args* a, double* out, int)
{
  ParamSource src;
  uint64_t    n = 0;
  forEachGeneratedVertex(t, a, [&](const VertexJob& job) {
    EvalOut o              = evalVertexD(a, job, src);
    out[3 * job.genIndex]     = o.v.x;
    out[3 * job.genIndex + 1] = o.v.y;
    out[3 * job.genIndex + 2] = o.v.z;
    n++;
  });
  return n;
}

uint64_t tco_generate_vertices_f64_params(const tco_table* t, const tc_frame_args* a, const double* const* positions,
                                          const double* const* normals, const double* const* texels, double* out)
{
  ParamSource src;
  src.positions = positions;
  src.normals   = normals;
  src.texels    = texels;
  uint64_t n    = 0;
  forEachGeneratedVertex(t, a, [&](const VertexJob& job) {
    EvalOut o              = evalVertexD(a, job, src);
    out[3 * job.genIndex]     = o.v.x;
    out[3 * job.genIndex + 1] = o.v.y;
    out[3 * job.genIndex + 2] = o.v.z;
    n++;
  });
  return n;
}

void tco_backward_f64(const tco_table* t, const tc_frame_args* a, const double* gradVertices, double* const* dPositions,
                      double* const* dNormals, double* const* dTexels)
{
  ParamSource src;
  forEachGeneratedVertex(t, a, [&](const VertexJob& job) {
    EvalOut o = evalVertexD(a, job, src);
    d3      g = {gradVertices[3 * job.genIndex], gradVertices[3 * job.genIndex + 1], gradVertices[3 * job.genIndex + 2]};
    if(dPositions && dPositions[job.inst])
      for(int k = 0; k < job.nBase; k++)
      {
        double* d = dPositions[job.inst] + 3 * job.vi[k];
        d[0] += job.w[k] * g.x;
        d[1] += job.w[k] * g.y;
        d[2] += job.w[k] * g.z;
      }
    if(!o.displaced)
      return;
    d3     m   = o.N * (1.0 / o.Nlen);
    double dh  = dotd(m, g);
    d3     dm  = g * o.h;
    d3     dN  = (dm - m * dotd(m, dm)) * (1.0 / o.Nlen);
    if(dNormals && dNormals[job.inst])
      for(int k = 0; k < job.nBase; k++)
      {
        d3 dn;
        if(job.nBase == 3)
        {
          d3 dnh = dN * job.w[k];
          dn     = (dnh - o.nhat[k] * dotd(o.nhat[k], dnh)) * (1.0 / o.nlen[k]);
        }
        else
          dn = dN;  // single normalisation: N == n, m == n/|n|
        double* d = dNormals[job.inst] + 3 * job.vi[k];
        d[0] += dn.x;
        d[1] += dn.y;
        d[2] += dn.z;
      }
    if(dTexels && dTexels[o.texIndex])
    {
      const tc_DisplacementTexture& tx = P<const tc_DisplacementTexture>(a->textures)[o.texIndex];
      double*                       T  = dTexels[o.texIndex];
      double                        dB = dh * o.s;
      T[(size_t)o.taps.y0 * tx.width + o.taps.x0] += o.taps.w00 * dB;
      T[(size_t)o.taps.y0 * tx.width + o.taps.x1] += o.taps.w10 * dB;
      T[(size_t)o.taps.y1 * tx.width + o.taps.x0] += o.taps.w01 * dB;
      T[(size_t)o.taps.y1 * tx.width + o.taps.x1] += o.taps.w11 * dB;
    }
  });
}

}  // extern "C"
