// ref_shader_pin.cpp — pins the oracle's restatement to the reference's own
// code, compiled here.
//
// TEST INFRASTRUCTURE (oracle side; built by oracle/Makefile target `ref` into
// oracle/_ref/, run by tests/test_ref_pin.py). Three things are compiled from
// the reference checkout unchanged or by a syntax-only rewrite:
//   - shaders/shaderio.h (with shaderio_core/scene/building.h) as C++ over
//     oracle/ref_shim/glsl_shim.h: every field of the pinned structs must have
//     the offset and size of the same field of include/tc_tessellation.h
//     (static_asserts generated by oracle/layout_pins.py; compiling is the
//     check);
//   - src/tessellation_table_nv_raw.hpp: the table every function below reads;
//   - shaders/tessellation.glsl:28-201, culling.glsl:27-92 and
//     displacement.glsl:27-120, rewritten by oracle/glsl_to_cpp.py (parameter
//     qualifiers, swizzle calls, float literal suffixes) into namespaces ref*.
// main() then runs every pinned shader function of the reference and the
// oracle's counterpart (tc_oracle.h) on exhaustive and seeded inputs and
// prints one JSON line per function: how many inputs were compared, how many
// differ (bit for bit, or beyond a stated tolerance where GLSL leaves the
// built-in's precision open: pow in the PN evaluation, normalize in the
// ripple), and the largest difference seen.
#include <algorithm>
#include <cinttypes>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "glsl_shim.h"

// the shader define the renderer passes (src/renderer_raytrace_clusters_tess.cpp:120:
// TessellationTable::m_maxSizeConfigs, 16); the GLSL side of shaderio_scene.h:41-43 has the same default
#define TESSTABLE_LOOKUP_SIZE 16

#include "shaderio.h"

#include "tc_oracle.h"

#include TC_REF_TABLE_HEADER

#include "layout_pins.inl"

// The globals the shader files read: the SceneBuilding UBO (`build`), the
// frame constants (`view`, `viewLast`) and the tessellation table UBO, whose
// arrays are buffer references (`.d[]`).
shaderio::SceneBuilding  build;
shaderio::FrameConstants view, viewLast;
struct RefTessTable
{
  struct
  {
    const shaderio::TessTableEntry* d;
  } entries;
  struct
  {
    const uint32_t* d;
  } vertices, triangles;
} tessTable;

namespace ref {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
#include "culling_glsl.inl"
#include "displacement_glsl.inl"
}  // namespace ref

// tess_getSplitFactor for every TESS_MAX_SPLIT_FACTOR the renderer allows
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 2
namespace ref_sf2 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf2
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 3
namespace ref_sf3 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf3
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 4
namespace ref_sf4 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf4
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 5
namespace ref_sf5 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf5
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 6
namespace ref_sf6 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf6
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 7
namespace ref_sf7 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf7
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 9
namespace ref_sf9 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf9
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 10
namespace ref_sf10 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf10
#undef TESS_MAX_SPLIT_FACTOR
#define TESS_MAX_SPLIT_FACTOR 11
namespace ref_sf11 {
using namespace glm;
using namespace shaderio;
#include "tessellation_glsl.inl"
}  // namespace ref_sf11

namespace {

typedef glm::uvec3 (*SplitFn)(glm::uvec3);

// ---------------------------------------------------------------------------
// reporting
// ---------------------------------------------------------------------------

struct Check
{
  std::string name;
  uint64_t    compared   = 0;
  uint64_t    mismatches = 0;
  double      maxErr     = 0.0;
  double      tolerance  = 0.0;  // 0: bit-exact
  std::string first;

  void miss(const std::string& what)
  {
    if(mismatches++ == 0)
      first = what;
  }
  void print() const
  {
    printf("{\"check\": \"%s\", \"compared\": %" PRIu64 ", \"mismatches\": %" PRIu64
           ", \"max_err\": %.9g, \"tolerance\": %.9g, \"first_mismatch\": \"%s\"}\n",
           name.c_str(), compared, mismatches, maxErr, tolerance, first.c_str());
    fflush(stdout);
  }
};

bool same_bits(float a, float b) { return std::memcmp(&a, &b, 4) == 0; }
bool same3(const glm::vec3& r, const float* o) { return same_bits(r.x, o[0]) && same_bits(r.y, o[1]) && same_bits(r.z, o[2]); }

std::string fmt3(const char* tag, const glm::vec3& r, const float* o)
{
  char b[256];
  snprintf(b, sizeof(b), "%s ref (%.9g %.9g %.9g) oracle (%.9g %.9g %.9g)", tag, r.x, r.y, r.z, o[0], o[1], o[2]);
  return b;
}

template <class F>
void parallel(uint32_t n, F&& fn)
{
  unsigned                 t = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for(unsigned i = 0; i < t; i++)
    pool.emplace_back([&, i]() { fn(i, t); });
  for(auto& th : pool)
    th.join();
  (void)n;
}

float uniform(std::mt19937& g, float lo, float hi) { return std::uniform_real_distribution<float>(lo, hi)(g); }

glm::vec3 rvec(std::mt19937& g, float s) { return {uniform(g, -s, s), uniform(g, -s, s), uniform(g, -s, s)}; }

// ---------------------------------------------------------------------------
// tessellation.glsl
// ---------------------------------------------------------------------------

Check check_encode(uint32_t n, uint32_t seed)
{
  Check        c;
  c.name = "tess_encodeBarycentrics";
  std::mt19937 g(seed);
  for(uint32_t i = 0; i < n; i++)
  {
    glm::vec3 w;
    switch(i & 3)
    {
      case 0:  // a point of the triangle
      {
        float u = uniform(g, 0, 1), v = uniform(g, 0, 1);
        if(u + v > 1.0f)
          u = 1.0f - u, v = 1.0f - v;
        w = {1.0f - u - v, u, v};
        break;
      }
      case 1:  // three independent values
        w = {uniform(g, 0, 1), uniform(g, 0, 1), uniform(g, 0, 1)};
        break;
      case 2:  // coordinates within a few ulps of a rounding tie (k + 0.5) / 32768
      {
        for(int k = 0; k < 3; k++)
        {
          float t = (float(g() % 32768) + 0.5f) / 32768.0f;
          int   d = int(g() % 9) - 4;
          for(; d > 0; d--)
            t = std::nextafter(t, 2.0f);
          for(; d < 0; d++)
            t = std::nextafter(t, -1.0f);
          w[k] = t;
        }
        break;
      }
      default:  // a table vertex composed with a sub-triangle's corners (split children)
      {
        glm::vec3 corner[3];
        for(int k = 0; k < 3; k++)
        {
          uint32_t u = g() % 32769, v = g() % (32769 - u);
          corner[k]  = ref::tess_decodeBarycentrics(u | (v << 16));
        }
        const uint32_t tv = tessellation_table::vertices[g() % tessellation_table::max_vertices];
        w                 = ref::tess_interpolate(corner, ref::tess_decodeBarycentrics(tv));
        break;
      }
    }
    const uint32_t r = ref::tess_encodeBarycentrics(w);
    const uint32_t o = tco_encode_barycentrics(w.x, w.y, w.z);
    c.compared++;
    if(r != o)
    {
      char b[160];
      snprintf(b, sizeof(b), "w (%.9g %.9g %.9g): ref %08x oracle %08x", w.x, w.y, w.z, r, o);
      c.miss(b);
    }
  }
  return c;
}

Check check_decode(uint32_t randomSamples, uint32_t seed)
{
  Check c;
  c.name = "tess_decodeBarycentrics";
  std::vector<Check> part(16);
  // every encoding of a point of the triangle: u + v <= 32768
  parallel(32769, [&](unsigned t, unsigned nt) {
    Check& p = part[t];
    for(uint32_t u = t; u <= 32768; u += nt)
      for(uint32_t v = 0; u + v <= 32768; v++)
      {
        const uint32_t  e = u | (v << 16);
        const glm::vec3 r = ref::tess_decodeBarycentrics(e);
        float           o[3];
        tco_decode_barycentrics(e, o);
        p.compared++;
        if(!same3(r, o))
          p.miss(fmt3("decode", r, o));
      }
  });
  for(const Check& p : part)
  {
    c.compared += p.compared;
    if(p.mismatches && !c.mismatches)
      c.first = p.first;
    c.mismatches += p.mismatches;
  }
  // and arbitrary 32-bit words
  std::mt19937 g(seed);
  for(uint32_t i = 0; i < randomSamples; i++)
  {
    const uint32_t  e = g();
    const glm::vec3 r = ref::tess_decodeBarycentrics(e);
    float           o[3];
    tco_decode_barycentrics(e, o);
    c.compared++;
    if(!same3(r, o))
      c.miss(fmt3("decode", r, o));
  }
  return c;
}

Check check_factors(uint32_t n, uint32_t seed)
{
  Check        c;
  c.name = "tess_getTessFactors";
  std::mt19937 g(seed);
  const float  heights[] = {720.0f, 1080.0f, 2160.0f};
  const float  rates[]   = {1.0f / 8.0f, 1.0f / 4.0f, 1.0f, 1.0f / 2.5f, 1.0f / 1.5f};
  for(uint32_t i = 0; i < n; i++)
  {
    const float     scale = std::pow(10.0f, uniform(g, -3.0f, 3.0f));
    const glm::vec3 a = rvec(g, scale), b = a + rvec(g, scale * uniform(g, 0.001f, 1.0f)),
                    cc = a + rvec(g, scale * uniform(g, 0.001f, 1.0f));
    build.viewPos     = rvec(g, scale * 4.0f);
    view.nearPlane    = std::pow(10.0f, uniform(g, -3.0f, 0.0f)) * scale;
    view.viewportf.y  = heights[g() % 3];
    view.tessRate     = rates[g() % 5];
    const glm::vec3 r = ref::tess_getTessFactors(a, b, cc);
    const float     pa[3] = {a.x, a.y, a.z}, pb[3] = {b.x, b.y, b.z}, pc[3] = {cc.x, cc.y, cc.z};
    const float     vp[3] = {build.viewPos.x, build.viewPos.y, build.viewPos.z};
    uint32_t        o[3];
    tco_tess_factors(pa, pb, pc, vp, view.nearPlane, view.viewportf.y, view.tessRate, o);
    c.compared++;
    // the reference keeps the rounded, clamped factors as floats; callers convert with uvec3()
    const glm::uvec3 ru(r);
    if(ru.x != o[0] || ru.y != o[1] || ru.z != o[2] || float(ru.x) != r.x || float(ru.y) != r.y || float(ru.z) != r.z)
    {
      char b2[200];
      snprintf(b2, sizeof(b2), "ref (%.9g %.9g %.9g) oracle (%u %u %u)", r.x, r.y, r.z, o[0], o[1], o[2]);
      c.miss(b2);
    }
  }
  return c;
}

Check check_split_factor()
{
  Check         c;
  c.name = "tess_getSplitFactor";
  const SplitFn fns[12] = {nullptr, nullptr, ref_sf2::tess_getSplitFactor, ref_sf3::tess_getSplitFactor,
                           ref_sf4::tess_getSplitFactor, ref_sf5::tess_getSplitFactor, ref_sf6::tess_getSplitFactor,
                           ref_sf7::tess_getSplitFactor, ref::tess_getSplitFactor, ref_sf9::tess_getSplitFactor,
                           ref_sf10::tess_getSplitFactor, ref_sf11::tess_getSplitFactor};
  for(uint32_t sf = 2; sf <= 11; sf++)
    for(uint32_t f = 1; f <= 32768 + 64; f++)
    {
      const glm::uvec3 r = fns[sf](glm::uvec3(f, f, f));
      const uint32_t   o = tco_split_factor(f, sf);
      c.compared++;
      if(r.x != o || r.y != o || r.z != o)
      {
        char b[120];
        snprintf(b, sizeof(b), "split factor %u, factor %u: ref %u oracle %u", sf, f, r.x, o);
        c.miss(b);
      }
    }
  return c;
}

Check check_get_config()
{
  Check              c;
  c.name = "tess_getConfig";
  const uint32_t     perms[6][3] = {{7, 11, 13}, {7, 13, 11}, {11, 7, 13}, {11, 13, 7}, {13, 7, 11}, {13, 11, 7}};
  for(uint32_t x = 1; x < 16; x++)
    for(uint32_t y = 1; y < 16; y++)
      for(uint32_t z = 1; z < 16; z++)
        for(const auto& p : perms)
        {
          glm::uvec3     tv(p[0], p[1], p[2]);
          uint32_t       f[3] = {x, y, z}, otv[3] = {p[0], p[1], p[2]};
          const uint32_t r    = ref::tess_getConfig(glm::uvec3(x, y, z), tv);
          const uint32_t o    = tco_get_config(f, otv);
          c.compared++;
          if(r != o || tv.x != otv[0] || tv.y != otv[1] || tv.z != otv[2])
          {
            char b[160];
            snprintf(b, sizeof(b), "factors (%u %u %u): ref %u (%u %u %u) oracle %u (%u %u %u)", x, y, z, r, tv.x,
                     tv.y, tv.z, o, otv[0], otv[1], otv[2]);
            c.miss(b);
          }
        }
  return c;
}

void check_config_lookups(const tco_table& t, Check& tri, Check& vert, Check& counts)
{
  tri.name    = "tess_getConfigTriangleVertices";
  vert.name   = "tess_getConfigVertexBarycentrics";
  counts.name = "tess_getConfigTriangleCount/VertexCount";
  for(uint32_t idx = 0; idx < TC_TESSTABLE_LOOKUP_ENTRIES; idx++)
  {
    const tc_TessTableEntry& e = t.entries[idx];
    if(e.numTriangles == 0)
      continue;
    for(uint32_t flip = 0; flip < 2; flip++)
    {
      const uint32_t cfg = idx | (flip << 15);
      counts.compared++;
      if(ref::tess_getConfigTriangleCount(cfg) != e.numTriangles || ref::tess_getConfigVertexCount(cfg) != e.numVertices)
        counts.miss("config " + std::to_string(cfg));
      for(uint32_t k = 0; k < e.numTriangles; k++)
      {
        const glm::uvec3 r = ref::tess_getConfigTriangleVertices(cfg, k);
        uint32_t         o[3];
        tco_config_triangle(&t, cfg, k, o);
        tri.compared++;
        if(r.x != o[0] || r.y != o[1] || r.z != o[2])
          tri.miss("config " + std::to_string(cfg) + " triangle " + std::to_string(k));
      }
      for(uint32_t k = 0; k < e.numVertices; k++)
      {
        const glm::vec3 r = ref::tess_getConfigVertexBarycentrics(cfg, k);
        float           o[3];
        tco_config_vertex(&t, cfg, k, o);
        vert.compared++;
        if(!same3(r, o))
          vert.miss(fmt3(("config " + std::to_string(cfg)).c_str(), r, o));
      }
    }
  }
}

Check check_interpolate(uint32_t n, uint32_t seed)
{
  Check        c;
  c.name = "tess_interpolate";
  std::mt19937 g(seed);
  for(uint32_t i = 0; i < n; i++)
  {
    const float scale = std::pow(10.0f, uniform(g, -2.0f, 2.0f));
    glm::vec3   base[3] = {rvec(g, scale), rvec(g, scale), rvec(g, scale)};
    uint32_t    u = g() % 32769, v = g() % (32769 - u);
    glm::vec3   w = ref::tess_decodeBarycentrics(u | (v << 16));
    const glm::vec3 r = ref::tess_interpolate(base, w);
    float           b9[9] = {base[0].x, base[0].y, base[0].z, base[1].x, base[1].y, base[1].z, base[2].x, base[2].y, base[2].z};
    float           w3[3] = {w.x, w.y, w.z}, o[3];
    tco_interpolate3(b9, w3, o);
    c.compared++;
    if(!same3(r, o))
      c.miss(fmt3("interpolate", r, o));
  }
  return c;
}

// ---------------------------------------------------------------------------
// culling.glsl
// ---------------------------------------------------------------------------

glm::mat4 perspective_look(std::mt19937& g, float& vh)
{
  // a perspective projection (vertical fov, aspect, near, far) times a view matrix
  const float fov = uniform(g, 0.3f, 1.6f), aspect = uniform(g, 1.0f, 2.4f), zn = uniform(g, 0.01f, 1.0f),
              zf = zn * uniform(g, 100.0f, 10000.0f);
  const float f  = 1.0f / std::tan(fov * 0.5f);
  glm::mat4   P  = {};
  P[0][0]        = f / aspect;
  P[1][1]        = -f;  // Vulkan's flipped y
  P[2][2]        = zf / (zn - zf);
  P[2][3]        = -1.0f;
  P[3][2]        = zn * zf / (zn - zf);
  // view: rotation about y and x, then a translation
  const float a = uniform(g, -3.2f, 3.2f), b = uniform(g, -1.2f, 1.2f);
  glm::mat4   V = {};
  V[0]          = {std::cos(a), std::sin(a) * std::sin(b), -std::sin(a) * std::cos(b), 0.0f};
  V[1]          = {0.0f, std::cos(b), std::sin(b), 0.0f};
  V[2]          = {std::sin(a), -std::cos(a) * std::sin(b), std::cos(a) * std::cos(b), 0.0f};
  V[3]          = {uniform(g, -20, 20), uniform(g, -20, 20), uniform(g, -60, 0), 1.0f};
  vh            = float(360 + g() % 1800);
  return P * V;
}

void check_culling(uint32_t n, uint32_t seed, Check& fr, Check& size)
{
  fr.name   = "intersectFrustum";
  size.name = "intersectSize";
  std::mt19937 g(seed);
  tc_FrameConstants tcView;
  std::memset(&tcView, 0, sizeof(tcView));
  for(uint32_t i = 0; i < n; i++)
  {
    float vh;
    viewLast.viewProjMatrix = perspective_look(g, vh);
    viewLast.viewportf      = glm::vec2(vh * uniform(g, 1.0f, 2.0f), vh);
    std::memcpy(&tcView, &viewLast, sizeof(tcView));  // the layouts are pinned above
    glm::mat4 W    = {};
    const float s  = uniform(g, 0.2f, 3.0f);
    W[0]           = {s, 0, 0, 0};
    W[1]           = {0, s * uniform(g, 0.5f, 1.5f), 0, 0};
    W[2]           = {0, 0, s, 0};
    W[3]           = {uniform(g, -30, 30), uniform(g, -30, 30), uniform(g, -80, 10), 1.0f};
    const glm::vec3 lo = rvec(g, 2.0f), hi = lo + glm::vec3(uniform(g, 0, 3), uniform(g, 0, 3), uniform(g, 0, 3));
    glm::vec4 rmin, rmax;
    bool      rvalid = false;
    const bool rin   = ref::intersectFrustum(lo, hi, W, rmin, rmax, rvalid);
    float     omin[4], omax[4];
    int       ovalid = 0;
    const float lo3[3] = {lo.x, lo.y, lo.z}, hi3[3] = {hi.x, hi.y, hi.z};
    const int  oin     = tco_intersect_frustum(lo3, hi3, &W[0][0], &tcView, omin, omax, &ovalid);
    fr.compared++;
    bool same = (rin ? 1 : 0) == oin && (rvalid ? 1 : 0) == ovalid;
    for(int k = 0; k < 4; k++)
      same = same && same_bits(rmin[k], omin[k]) && same_bits(rmax[k], omax[k]);
    if(!same)
      fr.miss("box " + std::to_string(i));
    const bool rs = ref::intersectSize(rmin, rmax);
    const int  os = tco_intersect_size(omin, omax, &tcView);
    size.compared++;
    if((rs ? 1 : 0) != os)
      size.miss("box " + std::to_string(i));
  }
}

// ---------------------------------------------------------------------------
// displacement.glsl
// ---------------------------------------------------------------------------

Check check_pn(uint32_t n, uint32_t seed)
{
  Check        c;
  c.name      = "deform_setupPN+deform_getPN";
  c.tolerance = 2e-6;  // relative to the triangle's extent: GLSL leaves pow's precision open
  std::mt19937 g(seed);
  for(uint32_t i = 0; i < n; i++)
  {
    const float scale = std::pow(10.0f, uniform(g, -2.0f, 2.0f));
    glm::vec3   v[3]  = {rvec(g, scale), rvec(g, scale), rvec(g, scale)};
    glm::vec3   nrm[3];
    for(auto& q : nrm)
      q = glm::normalize(rvec(g, 1.0f));
    float u = uniform(g, 0, 1), w2 = uniform(g, 0, 1);
    if(u + w2 > 1.0f)
      u = 1.0f - u, w2 = 1.0f - w2;
    const glm::vec3 bary(u, w2, 1.0f - u - w2);
    ref::DeformBasePN basis;
    ref::deform_setupPN(basis, v, nrm);
    const glm::vec3 r = ref::deform_getPN(basis, bary);
    float v9[9] = {v[0].x, v[0].y, v[0].z, v[1].x, v[1].y, v[1].z, v[2].x, v[2].y, v[2].z};
    float n9[9] = {nrm[0].x, nrm[0].y, nrm[0].z, nrm[1].x, nrm[1].y, nrm[1].z, nrm[2].x, nrm[2].y, nrm[2].z};
    float b3[3] = {bary.x, bary.y, bary.z}, o[3];
    tco_pn_position(v9, n9, b3, o);
    float extent = 0.0f;
    for(int k = 0; k < 3; k++)
      extent = std::max({extent, std::fabs(v[k].x), std::fabs(v[k].y), std::fabs(v[k].z)});
    double err = 0.0;
    for(int k = 0; k < 3; k++)
      err = std::max(err, (double)std::fabs(r[k] - o[k]) / extent);
    c.compared++;
    c.maxErr = std::max(c.maxErr, err);
    if(!(err <= c.tolerance))
      c.miss(fmt3("pn", r, o));
  }
  return c;
}

Check check_ripple(uint32_t n, uint32_t seed)
{
  Check        c;
  c.name      = "rippleDeform";
  // relative to the displaced vertex's magnitude (a few ulps of the result): GLSL defines
  // normalize(x) as x / length(x), the oracle multiplies by 1 / length(x)
  c.tolerance = 1e-6;
  std::mt19937 g(seed);
  tc_FrameConstants tcView;
  for(uint32_t i = 0; i < n; i++)
  {
    view.animationRippleFrequency = uniform(g, 1.0f, 30.0f);
    view.animationRippleAmplitude = uniform(g, 0.001f, 0.1f);
    view.animationRippleSpeed     = uniform(g, 0.1f, 4.0f);
    view.animationState           = uniform(g, 0.0f, 100.0f);
    std::memcpy(&tcView, &view, sizeof(tcView));
    const float     size = std::pow(10.0f, uniform(g, -1.0f, 2.0f));
    const glm::vec3 p    = rvec(g, size);
    const uint32_t  seedI = g() % 4096;
    const glm::vec3 r     = ref::rippleDeform(p, seedI, size);
    const float     p3[3] = {p.x, p.y, p.z};
    float           o[3];
    tco_ripple(p3, seedI, size, &tcView, o);
    const double mag = std::max({(double)std::fabs(r.x), (double)std::fabs(r.y), (double)std::fabs(r.z),
                                 (double)view.animationRippleAmplitude * size});
    double       err = 0.0;
    for(int k = 0; k < 3; k++)
      err = std::max(err, (double)std::fabs(r[k] - o[k]) / mag);
    c.compared++;
    c.maxErr = std::max(c.maxErr, err);
    if(!(err <= c.tolerance))
      c.miss(fmt3("ripple", r, o));
  }
  return c;
}

}  // namespace

int main(int argc, char** argv)
{
  // sample counts scale with argv[1] (1 = the default, a few seconds)
  const double   k    = argc > 1 ? std::max(0.01, atof(argv[1])) : 1.0;
  const uint32_t seed = argc > 2 ? (uint32_t)strtoul(argv[2], nullptr, 10) : 12345u;
  auto           N    = [&](double base) { return (uint32_t)std::max(1.0, base * k); };

  printf("{\"layout_fields\": %d, \"layout_structs\": %d}\n", TC_PINNED_FIELDS, TC_PINNED_STRUCTS);

  namespace tt = tessellation_table;
  static tco_table table;
  if(tco_table_init(&table, tt::vertices, tt::max_vertices, tt::triangles, tt::max_triangles, tt::configs,
                    tt::max_configs, tt::max_edge_segments)
     != 0)
  {
    fprintf(stderr, "tco_table_init failed on the reference table\n");
    return 1;
  }
  tessTable.entries.d   = reinterpret_cast<const shaderio::TessTableEntry*>(table.entries);
  tessTable.vertices.d  = tt::vertices;
  tessTable.triangles.d = tt::triangles;

  std::vector<Check> all;
  all.push_back(check_encode(N(4e6), seed));
  all.push_back(check_decode(N(1.6e7), seed + 1));
  all.push_back(check_factors(N(2e6), seed + 2));
  all.push_back(check_split_factor());
  all.push_back(check_get_config());
  {
    Check tri, vert, counts;
    check_config_lookups(table, tri, vert, counts);
    all.push_back(tri);
    all.push_back(vert);
    all.push_back(counts);
  }
  all.push_back(check_interpolate(N(1e6), seed + 3));
  {
    Check fr, sz;
    check_culling(N(1e6), seed + 4, fr, sz);
    all.push_back(fr);
    all.push_back(sz);
  }
  all.push_back(check_pn(N(1e6), seed + 5));
  all.push_back(check_ripple(N(1e6), seed + 6));
  int bad = 0;
  for(const Check& c : all)
  {
    c.print();
    bad += c.mismatches != 0;
  }
  return bad ? 1 : 0;
}
