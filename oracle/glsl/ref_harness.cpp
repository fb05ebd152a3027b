// ref_harness.cpp -- runs the reference's splat shaders on the host in the engine's dispatch order.
//
// TEST INFRASTRUCTURE ONLY: the executable reference that pins oracle/cpu_ref.c.  The shader bodies
// come from the reference checkout through oracle/glsl/make_ref.py (never committed); this file is the
// "driver + GPU" around them:
//
//   * parse_ply.comp for every splat (splat_load_thread.cc:114-135 supplies the 60-word offset table);
//   * per frame (engine.cc:1164-1290): the visible counter is zeroed (1167), rank.comp runs over all
//     splats, the key/index pairs are sorted (vrdxCmdSortKeyValueIndirect, 1218-1219: an ascending
//     32-bit radix sort, stable, restated here as std::stable_sort), the inverse map is filled with -1
//     (1226) and inverse_index.comp scatters it, then projection.comp writes the instances and the
//     indirect-draw words;
//   * the draw (DrawNormalPass, engine.cc:1380-1498): splat.vert for the 4 vertices of each visible
//     splat, the index pattern 4i + {0,1,2, 2,1,3} (engine.cc:606-616), Vulkan rasterisation of the
//     triangles (8 sub-pixel bits, pixel centres at +0.5, back faces culled with CCW front faces,
//     graphics_pipeline.cc:67-81), splat.frag per covered pixel, the depth test LESS against the
//     cleared 1.0 (or a caller depth) without depth writes, and the blend SRC_ALPHA /
//     ONE_MINUS_SRC_ALPHA for colour and alpha (engine.cc:281-291) over the clear (0, 0, 0, 1)
//     (engine.cc:1382-1387), with the fragment colour clamped to [0, 1] as the B8G8R8A8_UNORM
//     attachment does.
//
// Invocations run one at a time in ascending invocation index, so rank.comp's atomicAdd hands out
// slots in splat-id order: of the orders a GPU's atomics can produce, the one whose ties stay in
// ascending id after the stable sort.
#include "glsl.hpp"

namespace sh_parse_ply {
using namespace glsl;
uvec3 gl_GlobalInvocationID, gl_LocalInvocationID;
#include "parse_ply_comp.inc"
}  // namespace sh_parse_ply

namespace sh_rank {
using namespace glsl;
uvec3 gl_GlobalInvocationID, gl_LocalInvocationID;
#include "rank_comp.inc"
}  // namespace sh_rank

namespace sh_inverse_index {
using namespace glsl;
uvec3 gl_GlobalInvocationID, gl_LocalInvocationID;
#include "inverse_index_comp.inc"
}  // namespace sh_inverse_index

namespace sh_projection {
using namespace glsl;
uvec3 gl_GlobalInvocationID, gl_LocalInvocationID;
#include "projection_comp.inc"
}  // namespace sh_projection

namespace sh_vert {
using namespace glsl;
int gl_VertexIndex;
vec4 gl_Position;
#include "splat_vert.inc"
}  // namespace sh_vert

namespace sh_frag {
using namespace glsl;
#include "splat_frag.inc"
}  // namespace sh_frag

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

namespace {

constexpr uint32_t kGroup = 256;  // local_size_x of every compute shader

uint32_t groups(uint32_t n) { return (n + kGroup - 1) / kGroup; }

glsl::mat4 mat4_of(const float* p) {  // column-major float[16]
  glsl::mat4 m;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) m[c][r] = p[4 * c + r];
  return m;
}

}  // namespace

extern "C" {

// parse_ply.comp over n rows of the PLY body (row stride = offsets[59] floats).
void ref_parse_ply(const float* ply, uint32_t n, const uint32_t offsets[60], float* position, float* cov3d,
                   float* opacity, uint16_t* sh) {
  namespace S = sh_parse_ply;
  S::point_count = n;
  for (int i = 0; i < 60; ++i) S::offsets[i] = offsets[i];
  S::ply = const_cast<float*>(ply);
  S::gaussian_position = position;
  S::gaussian_cov3d = cov3d;
  S::gaussian_opacity = opacity;
  S::gaussian_sh = reinterpret_cast<glsl::float16_t*>(sh);
  for (uint32_t g = 0; g < groups(n); ++g) {
    // every invocation's part before barrier() first: the shared copy of the offset table
    for (uint32_t l = 0; l < 60; ++l) S::local_offsets[l] = S::offsets[l];
    for (uint32_t l = 0; l < kGroup; ++l) {
      S::gl_LocalInvocationID.x = l;
      S::gl_GlobalInvocationID.x = g * kGroup + l;
      S::shader_main();
    }
  }
}

// One frame's compute passes.  key/index: n entries (the first V are written, sorted);
// instance: V x 12 floats in sorted order; draw_indirect: the 12-word DrawIndirect buffer.
// Returns V.
uint32_t ref_frame_compute(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                           uint32_t n, const float* projection, const float* view, const float* model,
                           const float* eye, uint32_t width, uint32_t height, uint32_t* key, uint32_t* index,
                           float* instance, uint32_t* draw_indirect) {
  // rank.comp
  {
    namespace S = sh_rank;
    S::projection = mat4_of(projection);
    S::view = mat4_of(view);
    S::model = mat4_of(model);
    S::camera_position = glsl::vec3(eye[0], eye[1], eye[2]);
    S::screen_size.x = width;
    S::screen_size.y = height;
    S::point_count = n;
    S::gaussian_position = const_cast<float*>(position);
    S::visible_point_count = 0;
    S::key = key;
    S::index = index;
    for (uint32_t i = 0; i < groups(n) * kGroup; ++i) {
      S::gl_GlobalInvocationID.x = i;
      S::shader_main();
    }
  }
  const uint32_t v = sh_rank::visible_point_count;

  // vrdxCmdSortKeyValueIndirect: ascending keys, values carried, equal keys in their input order
  {
    std::vector<std::pair<uint32_t, uint32_t>> kv(v);
    for (uint32_t i = 0; i < v; ++i) kv[i] = {key[i], index[i]};
    std::stable_sort(kv.begin(), kv.end(),
                     [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                       return a.first < b.first;
                     });
    for (uint32_t i = 0; i < v; ++i) key[i] = kv[i].first, index[i] = kv[i].second;
  }

  // inverse map: fill(-1), then inverse_index.comp over the visible count
  std::vector<int> inverse(n ? n : 1, -1);
  {
    namespace S = sh_inverse_index;
    S::visible_point_count = v;
    S::index = index;
    S::inverse_index = inverse.data();
    for (uint32_t i = 0; i < groups(v) * kGroup; ++i) {
      S::gl_GlobalInvocationID.x = i;
      S::shader_main();
    }
  }

  // projection.comp over all splats
  {
    namespace S = sh_projection;
    S::projection = mat4_of(projection);
    S::view = mat4_of(view);
    S::model = mat4_of(model);
    S::camera_position = glsl::vec3(eye[0], eye[1], eye[2]);
    S::screen_size.x = width;
    S::screen_size.y = height;
    S::point_count = n;
    S::gaussian_position = const_cast<float*>(position);
    S::gaussian_cov3d = const_cast<float*>(cov3d);
    S::gaussian_opacity = const_cast<float*>(opacity);
    S::gaussian_sh = reinterpret_cast<glsl::f16vec4*>(const_cast<uint16_t*>(sh));
    S::instances = reinterpret_cast<glsl::vec4*>(instance);
    S::visible_point_count = v;
    S::inverse_map = inverse.data();
    for (uint32_t i = 0; i < groups(n) * kGroup; ++i) {
      S::gl_GlobalInvocationID.x = i;
      S::shader_main();
    }
    if (draw_indirect) {
      const uint32_t words[12] = {S::indexCount,   S::instanceCount,  S::firstIndex,  (uint32_t)S::vertexOffset,
                                  S::firstInstance, 0,                0,              0,
                                  S::vertexCount1, S::instanceCount1, S::firstVertex1, S::firstInstance1};
      std::memcpy(draw_indirect, words, sizeof words);
    }
  }
  return v;
}

// The draw: splat.vert + rasterisation + splat.frag + depth test + blend, instances in sorted order.
// image: H x W x 4 floats (RGBA, row 0 = framebuffer y 0), initialised here to the clear colour.
// unorm8 != 0 stores every blend result in the 8-bit attachment (round to nearest).  Returns the
// number of fragments that passed the depth test.
uint64_t ref_draw(const float* instance, uint32_t v, uint32_t width, uint32_t height, const float* depth_in,
                  int unorm8, float* image) {
  for (size_t i = 0; i < (size_t)width * height; ++i) {
    image[4 * i + 0] = 0.0f;
    image[4 * i + 1] = 0.0f;
    image[4 * i + 2] = 0.0f;
    image[4 * i + 3] = 1.0f;
  }
  sh_vert::instances = reinterpret_cast<glsl::vec4*>(const_cast<float*>(instance));
  constexpr int64_t kSub = 256;  // 8 sub-pixel bits
  const auto q8 = [](float x) {
    const float c = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return __builtin_nearbyintf(c * 255.0f) / 255.0f;
  };
  uint64_t frags = 0;
  struct Vtx {
    int64_t x, y;  // framebuffer position in 1/256 pixel
    float z;
    glsl::vec4 color;
    glsl::vec2 pos;
    bool ok;
  };
  const int tri[2][3] = {{0, 1, 2}, {2, 1, 3}};
  for (uint32_t i = 0; i < v; ++i) {
    Vtx q[4];
    for (int k = 0; k < 4; ++k) {
      sh_vert::gl_VertexIndex = (int)(4 * i + (uint32_t)k);
      sh_vert::shader_main();
      const glsl::vec4 p = sh_vert::gl_Position;  // w = 1: clip = NDC
      // viewport transform (x, y, width, height) = (0, 0, W, H), depth range [0, 1]
      const double xf = 0.5 * (double)width * (double)p.x + 0.5 * (double)width;
      const double yf = 0.5 * (double)height * (double)p.y + 0.5 * (double)height;
      q[k].ok = p.x == p.x && p.y == p.y && p.z == p.z && xf > -1e12 && xf < 1e12 && yf > -1e12 && yf < 1e12;
      q[k].x = q[k].ok ? (int64_t)__builtin_llround(xf * kSub) : 0;
      q[k].y = q[k].ok ? (int64_t)__builtin_llround(yf * kSub) : 0;
      q[k].z = p.z;
      q[k].color = sh_vert::out_color;
      q[k].pos = sh_vert::out_position;
    }
    for (const auto& t : tri) {
      const Vtx& a = q[t[0]];
      const Vtx& b = q[t[1]];
      const Vtx& c = q[t[2]];
      if (!(a.ok && b.ok && c.ok)) continue;  // NaN positions: no primitive
      // clip volume 0 <= z <= w (the quad's depth is constant)
      if (!(a.z >= 0.0f && a.z <= 1.0f && b.z >= 0.0f && b.z <= 1.0f && c.z >= 0.0f && c.z <= 1.0f)) continue;
      // twice the signed area in framebuffer coordinates (y down); Vulkan's a = -area2 / 2 > 0 is
      // counter-clockwise = front facing; back faces are culled
      const __int128 area2 = (__int128)(b.x - a.x) * (c.y - a.y) - (__int128)(b.y - a.y) * (c.x - a.x);
      if (area2 >= 0) continue;
      // orient so that the interior has positive edge functions: traverse a, c, b
      const Vtx* vv[3] = {&a, &c, &b};
      int64_t xmin = std::min({a.x, b.x, c.x}), xmax = std::max({a.x, b.x, c.x});
      int64_t ymin = std::min({a.y, b.y, c.y}), ymax = std::max({a.y, b.y, c.y});
      // pixels whose centre (px + 1/2) * 256 lies in [min, max]
      auto lo = [&](int64_t m) { return (m - kSub / 2 + kSub - 1) >= 0 ? (m - kSub / 2 + kSub - 1) / kSub : 0; };
      auto hi = [&](int64_t m) { return (m - kSub / 2) >= 0 ? (m - kSub / 2) / kSub : -1; };
      const int64_t px0 = std::max<int64_t>(0, lo(xmin)), px1 = std::min<int64_t>((int64_t)width - 1, hi(xmax));
      const int64_t py0 = std::max<int64_t>(0, lo(ymin)), py1 = std::min<int64_t>((int64_t)height - 1, hi(ymax));
      if (px0 > px1 || py0 > py1) continue;
      // edge e(k): from vv[k] to vv[k+1]; owns its boundary samples iff dy > 0 or (dy == 0 and dx > 0),
      // the complement of the reversed edge, so a sample on a shared edge is covered exactly once
      int64_t ex[3], ey[3];
      bool own[3];
      for (int k = 0; k < 3; ++k) {
        const Vtx* s = vv[k];
        const Vtx* e = vv[(k + 1) % 3];
        ex[k] = e->x - s->x;
        ey[k] = e->y - s->y;
        own[k] = ey[k] > 0 || (ey[k] == 0 && ex[k] > 0);
      }
      const double inv_area = 1.0 / (double)(-area2);
      for (int64_t py = py0; py <= py1; ++py) {
        const int64_t sy = py * kSub + kSub / 2;
        for (int64_t px = px0; px <= px1; ++px) {
          const int64_t sx = px * kSub + kSub / 2;
          __int128 w[3];
          bool in = true;
          for (int k = 0; k < 3 && in; ++k) {
            const Vtx* s = vv[k];
            // positive on the interior side for this orientation
            w[k] = (__int128)(sx - s->x) * ey[k] - (__int128)(sy - s->y) * ex[k];
            w[k] = -w[k];
            in = w[k] > 0 || (w[k] == 0 && own[k]);
          }
          if (!in) continue;
          const size_t pix = (size_t)py * width + (size_t)px;
          const float z = a.z;
          const float dref = depth_in ? depth_in[pix] : 1.0f;
          if (!(z < dref)) continue;
          ++frags;
          // barycentrics: w[k] is the weight of the vertex opposite edge k
          const double l0 = (double)w[1] * inv_area;  // vv[0] is opposite edge 1 (vv[1] -> vv[2])
          const double l1 = (double)w[2] * inv_area;
          const double l2 = (double)w[0] * inv_area;
          // w = 1 everywhere, so perspective-correct interpolation is linear in screen space
          glsl::vec2 p;
          p.x = (float)(l0 * vv[0]->pos.x + l1 * vv[1]->pos.x + l2 * vv[2]->pos.x);
          p.y = (float)(l0 * vv[0]->pos.y + l1 * vv[1]->pos.y + l2 * vv[2]->pos.y);
          // the four vertices carry the same colour, which interpolates to itself
          sh_frag::color = a.color;
          sh_frag::position = p;
          sh_frag::shader_main();
          const glsl::vec4 o = sh_frag::out_color;
          const auto clamp01 = [](float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); };
          const float sa = clamp01(o.a), sr = clamp01(o.r), sg = clamp01(o.g), sb = clamp01(o.b);
          float* d = image + 4 * pix;
          const float ia = 1.0f - sa;
          float r = sr * sa + d[0] * ia, g = sg * sa + d[1] * ia, bb = sb * sa + d[2] * ia, al = sa * sa + d[3] * ia;
          if (unorm8) r = q8(r), g = q8(g), bb = q8(bb), al = q8(al);
          d[0] = r, d[1] = g, d[2] = bb, d[3] = al;
        }
      }
    }
  }
  return frags;
}

}  // extern "C"
