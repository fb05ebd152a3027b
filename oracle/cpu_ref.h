/*
 * cpu_ref.h -- CPU oracle for the vkgs per-frame splat pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (vkgs_gb300/) links, loads
 * or calls this library; only tests/, the smoke check and the CPU-baseline arm
 * of bench.py do, and only as the checker / the timed CPU reference.
 *
 * Parity status: PINNED to the reference's shaders executed on the host
 * (oracle/glsl/: the shader bodies compiled against a C++ GLSL subset; checked
 * by tests/test_ref_pin.py and tests/golden/ref_fixtures.json).  This file is a
 * scalar restatement of the reference shaders with every floating-point
 * operation order pinned (GLSL column-major, left-to-right sums, no FMA
 * contraction: build with -ffp-contract=off); its visible set, keys, sorted
 * order, ndc, colour and opacity equal the shaders' bit for bit.
 *
 * Matrices are column-major float[16] exactly like glm::mat4: m[col*4 + row].
 */
#ifndef VKGS_ORACLE_CPU_REF_H
#define VKGS_ORACLE_CPU_REF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The Camera uniform (src/vkgs/vulkan/shader/uniforms.h:10-15) plus the model
 * push constant (src/shader/rank.comp:13). */
typedef struct or_camera {
  float projection[16];
  float view[16];
  float model[16];
  float eye[3];
  uint32_t width;
  uint32_t height;
} or_camera;

/* ---- A1: camera math (src/vkgs/scene/camera.cc:25-45) ---- */
void or_perspective_vk(float fovy, float aspect, float znear, float zfar, float out[16]);
void or_look_at(const float eye[3], const float center[3], const float up[3], float out[16]);
void or_orbit_eye(const float center[3], float r, float phi, float theta, float out[3]);
void or_mat4_mul(const float a[16], const float b[16], float out[16]);

/* ---- A3: parse_ply.comp activation (src/shader/parse_ply.comp:34-97) ---- */
uint16_t or_f32_to_f16(float f);
float or_f16_to_f32(uint16_t h);
void or_parse_ply(const float* ply, uint32_t n, const uint32_t offsets[60], float* position, float* cov3d,
                  float* opacity, uint16_t* sh);

/* ---- A4: rank.comp cull + key + compaction in id order (src/shader/rank.comp:27-41) ---- */
uint32_t or_rank(const float* position, uint32_t n, const or_camera* cam, uint32_t* key, uint32_t* index);

/* ---- A5: stable ascending key/value sort (vulkan_radix_sort semantics, engine.cc:1218-1219) ---- */
void or_sort_kv(uint32_t* key, uint32_t* value, uint32_t n);

/* ---- A6: projection.comp for the sorted visible list (src/shader/projection.comp:60-179) ----
 * instance: V x 12 floats in the reference layout {ndc.xyz, 0}, {rot_scale col0, col1}, {rgb, opacity}.
 * record:   V x 16 floats, the raster record {cx, cy, M00, M01}, {M10, M11, cz, o}, {r', g', b', 0},
 *           {hx, hy, 0, 0} where M = rot_scale^-1, rgb' = min(rgb, 1) and hx < 0 marks "not drawn". */
void or_project(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                const uint32_t* sorted_index, uint32_t v, const or_camera* cam, float* instance, float* record);

/* ---- A7+A8: quad coverage + back-to-front SRC_ALPHA/ONE_MINUS_SRC_ALPHA blend ----
 * image: H x W x 4 floats (RGBA, row 0 = top).  depth_in: optional H x W depth (NULL = cleared 1.0).
 * unorm8 != 0 emulates the B8G8R8A8_UNORM framebuffer (quantise after every blend).
 * Returns the fragment count F (pixel centre inside the 3-sigma quad and depth test passed). */
uint64_t or_raster(const float* record, uint32_t v, uint32_t width, uint32_t height, const float* depth_in,
                   int unorm8, float* image);

/* Same, restricted to the 16-row bands b with b % band_stride == band_offset (a bounded sample of the
 * blend for timing; the other rows keep the clear colour). */
uint64_t or_raster_bands(const float* record, uint32_t v, uint32_t width, uint32_t height, const float* depth_in,
                         int unorm8, uint32_t band_stride, uint32_t band_offset, float* image);

/* Whole FP32 frame: A4 -> A5 -> A6 -> A7/A8.  Returns the visible count; fills key/index (sorted),
 * instance (V x 12, may be NULL), image, *fragments. */
uint32_t or_render_frame(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                         uint32_t n, const or_camera* cam, const float* depth_in, int unorm8, uint32_t* key,
                         uint32_t* index, float* instance, float* image, uint64_t* fragments);

/* FP64 twin of the whole frame with the literal reference formulas (atan2/cos/sin, exp) evaluated in
 * double.  image: H x W x 4 doubles.  Returns the FP64 visible count. */
uint32_t or_render_frame_f64(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                             uint32_t n, const or_camera* cam, double* image);

int or_num_threads(void);
void or_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#endif
