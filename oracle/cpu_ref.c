/*
 * cpu_ref.c -- CPU oracle for the vkgs per-frame splat pipeline.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU-baseline
 * arm of bench.py as the checker.  The product never links or calls it.
 *
 * Parity status: PINNED to the reference's own shaders.  The reference ships no
 * tests, fixtures or CPU code, and its shaders need a Vulkan stack that does
 * not exist here, so oracle/glsl/ compiles the shader bodies themselves for the
 * host (a C++ GLSL subset + a harness that dispatches them in the engine's
 * order and rasterises the quads with Vulkan's rules); tests/test_ref_pin.py
 * compares this file with them (live where the reference checkout exists,
 * through tests/golden/ref_fixtures.json everywhere): parse_ply, visible set,
 * keys, order, ndc, colour and opacity bit-exact, rot_scale within 4 x 2^-24 of
 * its column norm, images within 1/255 but for quad-edge coverage flips.  This
 * is a scalar restatement of the reference shaders; each function cites the
 * shader lines it follows.  Build with -O2 -ffp-contract=off -fno-fast-math so
 * that every product/sum below is one IEEE-754 binary32 rounding, evaluated in
 * GLSL order (column-major, left-to-right sums).
 *
 * Two deliberate definitions where GLSL leaves the result to the driver:
 *   - normalize(v) = v / sqrt(dot(v, v)) with correctly rounded sqrt and divide;
 *   - the eigen-angle of projection.comp:128-132 (theta = atan2(s2t, c2t)/2,
 *     cos(theta), sin(theta)) is evaluated with the exact half-angle identities
 *     using only sqrt/divide, so CPU and GPU produce identical bits.  The FP64
 *     twin (or_render_frame_f64) uses the literal atan2/cos/sin in double.
 */
#include "cpu_ref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define M4(m, c, r) ((m)[(c)*4 + (r)])
#define M3(m, c, r) ((m)[(c)*3 + (r)])
#define M2(m, c, r) ((m)[(c)*2 + (r)])

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------- */
/* A1: camera (src/vkgs/scene/camera.cc:25-45), glm formulas restated.        */
/* ------------------------------------------------------------------------- */

/* glm mat4 * mat4: column j = a[0]*b[j][0] + a[1]*b[j][1] + a[2]*b[j][2] + a[3]*b[j][3]. */
void or_mat4_mul(const float a[16], const float b[16], float out[16]) {
  float r[16];
  for (int j = 0; j < 4; ++j)
    for (int i = 0; i < 4; ++i)
      M4(r, j, i) = ((M4(a, 0, i) * M4(b, j, 0) + M4(a, 1, i) * M4(b, j, 1)) + M4(a, 2, i) * M4(b, j, 2)) +
                    M4(a, 3, i) * M4(b, j, 3);
  memcpy(out, r, sizeof(r));
}

/* glm::perspective (right-handed, clip z in [-1,1]) then the gl->vulkan conversion of camera.cc:29-34. */
void or_perspective_vk(float fovy, float aspect, float znear, float zfar, float out[16]) {
  float p[16];
  memset(p, 0, sizeof(p));
  const float t = tanf(fovy / 2.0f);
  M4(p, 0, 0) = 1.0f / (aspect * t);
  M4(p, 1, 1) = 1.0f / t;
  M4(p, 2, 2) = -(zfar + znear) / (zfar - znear);
  M4(p, 2, 3) = -1.0f;
  M4(p, 3, 2) = -(2.0f * zfar * znear) / (zfar - znear);
  float conv[16];
  memset(conv, 0, sizeof(conv));
  M4(conv, 0, 0) = 1.0f;
  M4(conv, 1, 1) = -1.0f;
  M4(conv, 2, 2) = 0.5f;
  M4(conv, 3, 2) = 0.5f;
  M4(conv, 3, 3) = 1.0f;
  or_mat4_mul(conv, p, out);
}

static float dot3f(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static void cross3f(const float x[3], const float y[3], float out[3]) {
  out[0] = x[1] * y[2] - y[1] * x[2];
  out[1] = x[2] * y[0] - y[2] * x[0];
  out[2] = x[0] * y[1] - y[0] * x[1];
}

/* glm normalize: v * inversesqrt(dot(v, v)) with inversesqrt(x) = 1 / sqrt(x). */
static void glm_normalize3f(const float v[3], float out[3]) {
  const float inv = 1.0f / sqrtf(dot3f(v, v));
  out[0] = v[0] * inv;
  out[1] = v[1] * inv;
  out[2] = v[2] * inv;
}

/* glm::lookAt, right-handed (camera.cc:37 passes up = (0,1,0)). */
void or_look_at(const float eye[3], const float center[3], const float up[3], float out[16]) {
  float fd[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
  float f[3], s0[3], s[3], u[3];
  glm_normalize3f(fd, f);
  cross3f(f, up, s0);
  glm_normalize3f(s0, s);
  cross3f(s, f, u);
  memset(out, 0, 16 * sizeof(float));
  M4(out, 0, 0) = s[0];
  M4(out, 1, 0) = s[1];
  M4(out, 2, 0) = s[2];
  M4(out, 0, 1) = u[0];
  M4(out, 1, 1) = u[1];
  M4(out, 2, 1) = u[2];
  M4(out, 0, 2) = -f[0];
  M4(out, 1, 2) = -f[1];
  M4(out, 2, 2) = -f[2];
  M4(out, 3, 0) = -dot3f(s, eye);
  M4(out, 3, 1) = -dot3f(u, eye);
  M4(out, 3, 2) = dot3f(f, eye);
  M4(out, 3, 3) = 1.0f;
}

/* Camera::Eye (camera.cc:39-45): center + r * (sin phi sin theta, cos phi, sin phi cos theta). */
void or_orbit_eye(const float center[3], float r, float phi, float theta, float out[3]) {
  const float sp = sinf(phi), cp = cosf(phi), st = sinf(theta), ct = cosf(theta);
  const float d[3] = {sp * st, cp, sp * ct};
  out[0] = center[0] + r * d[0];
  out[1] = center[1] + r * d[1];
  out[2] = center[2] + r * d[2];
}

/* inverse(model) * vec4(eye, 1), divided by w (projection.comp:85-86).  Evaluated in double through
 * the adjugate and rounded once to float; exact for the identity model. */
static void camera_model_position(const or_camera* cam, float out[3]) {
  double m[16], inv[16];
  for (int i = 0; i < 16; ++i) m[i] = cam->model[i];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] +
           m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
           m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] +
           m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
            m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
           m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] +
           m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
           m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
            m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] +
           m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] -
           m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] +
            m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
            m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] -
           m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] +
           m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] -
            m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] +
            m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  const double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  const double e[4] = {cam->eye[0], cam->eye[1], cam->eye[2], 1.0};
  double p[4];
  for (int i = 0; i < 4; ++i) p[i] = (inv[i] * e[0] + inv[4 + i] * e[1] + inv[8 + i] * e[2] + inv[12 + i] * e[3]) / det;
  for (int i = 0; i < 3; ++i) out[i] = (float)(p[i] / p[3]);
}

/* ------------------------------------------------------------------------- */
/* A3: parse_ply.comp (src/shader/parse_ply.comp:34-97).                      */
/* ------------------------------------------------------------------------- */

/* IEEE binary32 -> binary16, round to nearest even (GLSL float16_t(x) conversion). */
uint16_t or_f32_to_f16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t ax = x & 0x7fffffffu;
  if (ax >= 0x7f800000u) {                      /* inf or nan */
    if (ax == 0x7f800000u) return (uint16_t)(sign | 0x7c00u);
    return (uint16_t)(sign | 0x7e00u | ((ax >> 13) & 0x3ffu));
  }
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* rounds to >= 65520 -> inf */
  if (ax >= 0x38800000u) {                      /* normal half */
    uint32_t mant = ax & 0x7fffffu;
    uint32_t exp = (ax >> 23) - 127 + 15;
    uint32_t h = (exp << 10) | (mant >> 13);
    const uint32_t rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1; /* carry may bump the exponent */
    return (uint16_t)(sign | h);
  }
  if (ax < 0x33000000u) return (uint16_t)sign;  /* below half of the smallest subnormal */
  /* subnormal half: value = m * 2^-24 */
  const uint32_t e = ax >> 23;                   /* biased float exponent, 102..112 */
  const uint32_t mant = (ax & 0x7fffffu) | 0x800000u;
  const uint32_t shift = 126 - e;                /* 14..24 */
  uint32_t h = mant >> shift;
  const uint32_t rem = mant & ((1u << shift) - 1u);
  const uint32_t half = 1u << (shift - 1);
  if (rem > half || (rem == half && (h & 1u))) h += 1;
  return (uint16_t)(sign | h);
}

float or_f16_to_f32(uint16_t h) {
  const uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu;
  uint32_t m = h & 0x3ffu;
  uint32_t x;
  if (e == 0x1fu) {
    x = sign | 0x7f800000u | (m << 13);
  } else if (e == 0) {
    if (m == 0) {
      x = sign;
    } else {
      int ee = -1;
      do {
        m <<= 1;
        ++ee;
      } while (!(m & 0x400u));
      x = sign | ((uint32_t)(127 - 15 - ee) << 23) | ((m & 0x3ffu) << 13);
    }
  } else {
    x = sign | ((e + 127 - 15) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &x, 4);
  return f;
}

void or_parse_ply(const float* ply, uint32_t n, const uint32_t off[60], float* position, float* cov3d,
                  float* opacity, uint16_t* sh) {
  const size_t base = off[59];
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)n; ++ii) {
    const size_t id = (size_t)ii;
    const float* row = ply + base * id;
    float s[3] = {expf(row[off[3]]), expf(row[off[4]]), expf(row[off[5]])};
    float q[4] = {row[off[6]], row[off[7]], row[off[8]], row[off[9]]};
    const float len = sqrtf(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
    for (int k = 0; k < 4; ++k) q[k] = q[k] / len;
    const float xx = q[0] * q[0], yy = q[1] * q[1], zz = q[2] * q[2];
    const float xy = q[0] * q[1], xz = q[0] * q[2], yz = q[1] * q[2];
    const float wx = q[3] * q[0], wy = q[3] * q[1], wz = q[3] * q[2];
    float rot[9];
    M3(rot, 0, 0) = 1.0f - 2.0f * (yy + zz);
    M3(rot, 0, 1) = 2.0f * (xy + wz);
    M3(rot, 0, 2) = 2.0f * (xz - wy);
    M3(rot, 1, 0) = 2.0f * (xy - wz);
    M3(rot, 1, 1) = 1.0f - 2.0f * (xx + zz);
    M3(rot, 1, 2) = 2.0f * (yz + wx);
    M3(rot, 2, 0) = 2.0f * (xz + wy);
    M3(rot, 2, 1) = 2.0f * (yz - wx);
    M3(rot, 2, 2) = 1.0f - 2.0f * (xx + yy);
    float ss[9];
    memset(ss, 0, sizeof(ss));
    M3(ss, 0, 0) = s[0] * s[0];
    M3(ss, 1, 1) = s[1] * s[1];
    M3(ss, 2, 2) = s[2] * s[2];
    /* cov3d = rot * ss * transpose(rot), evaluated as (rot * ss) * rot^T */
    float t[9], c[9];
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i)
        M3(t, j, i) = (M3(rot, 0, i) * M3(ss, j, 0) + M3(rot, 1, i) * M3(ss, j, 1)) + M3(rot, 2, i) * M3(ss, j, 2);
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i)
        M3(c, j, i) = (M3(t, 0, i) * M3(rot, 0, j) + M3(t, 1, i) * M3(rot, 1, j)) + M3(t, 2, i) * M3(rot, 2, j);
    float* cv = cov3d + 6 * id;
    cv[0] = M3(c, 0, 0);
    cv[1] = M3(c, 1, 0);
    cv[2] = M3(c, 2, 0);
    cv[3] = M3(c, 1, 1);
    cv[4] = M3(c, 2, 1);
    cv[5] = M3(c, 2, 2);
    position[3 * id + 0] = row[off[0]];
    position[3 * id + 1] = row[off[1]];
    position[3 * id + 2] = row[off[2]];
    for (int i = 0; i < 48; ++i) sh[48 * id + i] = or_f32_to_f16(row[off[10 + i]]);
    opacity[id] = 1.0f / (1.0f + expf(-row[off[58]]));
  }
}

/* ------------------------------------------------------------------------- */
/* A4: rank.comp (src/shader/rank.comp:27-41).                                */
/* ------------------------------------------------------------------------- */

static void mat4_vec4(const float m[16], const float v[4], float out[4]) {
  for (int i = 0; i < 4; ++i)
    out[i] = ((M4(m, 0, i) * v[0] + M4(m, 1, i) * v[1]) + M4(m, 2, i) * v[2]) + M4(m, 3, i) * v[3];
}

static int rank_one(const float* position, size_t id, const float pvm[16], uint32_t* key_out) {
  float p[4] = {position[3 * id + 0], position[3 * id + 1], position[3 * id + 2], 1.0f};
  float c[4];
  mat4_vec4(pvm, p, c);
  const float x = c[0] / c[3], y = c[1] / c[3], z = c[2] / c[3];
  if (fabsf(x) <= 1.0f && fabsf(y) <= 1.0f && z >= 0.0f && z <= 1.0f) {
    const float k = 1.0f - z;
    memcpy(key_out, &k, 4);
    return 1;
  }
  return 0;
}

/* The atomicAdd slot of rank.comp:38 is replaced by compaction in ascending id: the tie rule of this
 * implementation (equal keys stay in ascending splat id after the stable sort). */
uint32_t or_rank(const float* position, uint32_t n, const or_camera* cam, uint32_t* key, uint32_t* index) {
  float pv[16], pvm[16];
  or_mat4_mul(cam->projection, cam->view, pv);
  or_mat4_mul(pv, cam->model, pvm);
  const int nt = or_num_threads();
  const size_t chunk = ((size_t)n + (size_t)nt - 1) / (size_t)nt;
  uint32_t* counts = (uint32_t*)calloc((size_t)nt + 1, sizeof(uint32_t));
#pragma omp parallel num_threads(nt)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    const size_t b = chunk * (size_t)t, e = (b + chunk < n) ? b + chunk : n;
    uint32_t cnt = 0, k;
    for (size_t id = b; id < e; ++id) cnt += (uint32_t)rank_one(position, id, pvm, &k);
    counts[t + 1] = cnt;
#pragma omp barrier
#pragma omp single
    for (int i = 0; i < nt; ++i) counts[i + 1] += counts[i];
    uint32_t slot = counts[t];
    for (size_t id = b; id < e; ++id) {
      if (rank_one(position, id, pvm, &k)) {
        key[slot] = k;
        index[slot] = (uint32_t)id;
        ++slot;
      }
    }
  }
  const uint32_t v = counts[nt];
  free(counts);
  return v;
}

/* ------------------------------------------------------------------------- */
/* A5: stable ascending sort of 32-bit keys carrying 32-bit values.           */
/* ------------------------------------------------------------------------- */

void or_sort_kv(uint32_t* key, uint32_t* value, uint32_t n) {
  if (n < 2) return;
  uint32_t* k2 = (uint32_t*)malloc((size_t)n * 4);
  uint32_t* v2 = (uint32_t*)malloc((size_t)n * 4);
  uint32_t *ks = key, *vs = value, *kd = k2, *vd = v2;
  for (int pass = 0; pass < 4; ++pass) {
    const int shift = pass * 8;
    size_t cnt[257];
    memset(cnt, 0, sizeof(cnt));
    for (uint32_t i = 0; i < n; ++i) cnt[((ks[i] >> shift) & 0xffu) + 1]++;
    for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
    for (uint32_t i = 0; i < n; ++i) {
      const size_t pos = cnt[(ks[i] >> shift) & 0xffu]++;
      kd[pos] = ks[i];
      vd[pos] = vs[i];
    }
    uint32_t* t = ks;
    ks = kd;
    kd = t;
    t = vs;
    vs = vd;
    vd = t;
  }
  /* 4 passes: the result is back in the caller's arrays */
  free(k2);
  free(v2);
}

/* ------------------------------------------------------------------------- */
/* A6: projection.comp (src/shader/projection.comp:80-179).                   */
/* ------------------------------------------------------------------------- */

static void mat3_mul(const float a[9], const float b[9], float out[9]) {
  float r[9];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i)
      M3(r, j, i) = (M3(a, 0, i) * M3(b, j, 0) + M3(a, 1, i) * M3(b, j, 1)) + M3(a, 2, i) * M3(b, j, 2);
  memcpy(out, r, sizeof(r));
}

static void mat3_transpose(const float a[9], float out[9]) {
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) M3(out, j, i) = M3(a, i, j);
}

static void mat3_of_mat4(const float m[16], float out[9]) {
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) M3(out, j, i) = M4(m, j, i);
}

static void mat2_mul(const float a[4], const float b[4], float out[4]) {
  float r[4];
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) M2(r, j, i) = M2(a, 0, i) * M2(b, j, 0) + M2(a, 1, i) * M2(b, j, 1);
  memcpy(out, r, sizeof(r));
}

static float dot4f(const float a[4], const float b[4]) { return ((a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]) + a[3] * b[3]; }

/* cos(theta), sin(theta) for theta = atan2(s2t, c2t) / 2 through the half-angle identities
 * (theta lies in [-pi/2, pi/2], so cos >= 0 and sin carries the sign of s2t). */
static void half_angle(float s2t, float c2t, float* ct, float* st) {
  if (c2t >= 0.0f) {
    const float c = sqrtf(0.5f * (1.0f + c2t));
    *ct = c;
    *st = s2t / (2.0f * c);
  } else {
    const float s = sqrtf(0.5f * (1.0f - c2t));
    *st = copysignf(s, s2t);
    *ct = fabsf(s2t) / (2.0f * s);
  }
}

static void project_one(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                        uint32_t id, const or_camera* cam, const float cam_m[3], float lpx, float lpy,
                        float* inst, float* rec) {
  const float* cv = cov3d + 6 * (size_t)id;
  float pos[4] = {position[3 * (size_t)id + 0], position[3 * (size_t)id + 1], position[3 * (size_t)id + 2], 1.0f};

  /* dir = normalize(pos.xyz - camera_model_position.xyz) (projection.comp:85-87) */
  float d[3] = {pos[0] - cam_m[0], pos[1] - cam_m[1], pos[2] - cam_m[2]};
  const float dl = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
  const float dir[3] = {d[0] / dl, d[1] / dl, d[2] / dl};

  /* cov3d = mat3(v0, v0.y, v1.xy, v0.z, v1.yz) (projection.comp:80-92) */
  float cov[9] = {cv[0], cv[1], cv[2], cv[1], cv[3], cv[4], cv[2], cv[4], cv[5]};

  float m3[9], m3t[9], tmp[9];
  mat3_of_mat4(cam->model, m3);
  mat3_transpose(m3, m3t);
  mat3_mul(m3, cov, tmp);
  mat3_mul(tmp, m3t, cov);
  float p1[4];
  mat4_vec4(cam->model, pos, p1);

  mat3_of_mat4(cam->view, m3);
  mat3_transpose(m3, m3t);
  mat3_mul(m3, cov, tmp);
  mat3_mul(tmp, m3t, cov);
  float pv[4];
  mat4_vec4(cam->view, p1, pv);

  /* J (projection.comp:105-108) */
  const float r = sqrtf((pv[0] * pv[0] + pv[1] * pv[1]) + pv[2] * pv[2]);
  float J[9] = {-1.0f / pv[2], 0.0f, -2.0f * pv[0] / r,  0.0f, -1.0f / pv[2], -2.0f * pv[1] / r,
                pv[0] / pv[2] / pv[2], pv[1] / pv[2] / pv[2], -2.0f * pv[2] / r};
  float Jt[9];
  mat3_transpose(J, Jt);
  mat3_mul(J, cov, tmp);
  mat3_mul(tmp, Jt, cov);

  /* cov2d = mat2(projection) * mat2(cov3d) * mat2(projection) (projection.comp:111-112) */
  const float P2[4] = {M4(cam->projection, 0, 0), M4(cam->projection, 0, 1), M4(cam->projection, 1, 0),
                       M4(cam->projection, 1, 1)};
  const float C2[4] = {M3(cov, 0, 0), M3(cov, 0, 1), M3(cov, 1, 0), M3(cov, 1, 1)};
  float t2[4], c2[4];
  mat2_mul(P2, C2, t2);
  mat2_mul(t2, P2, c2);
  M2(c2, 0, 0) += lpx;
  M2(c2, 1, 1) += lpy;

  /* eigen decomposition (projection.comp:121-134) */
  const float a = M2(c2, 0, 0), b = M2(c2, 1, 1), c = M2(c2, 1, 0);
  const float D = sqrtf((a - b) * (a - b) + 4.0f * c * c);
  const float s0 = sqrtf(0.5f * (a + b + D));
  const float s1 = sqrtf(0.5f * (a + b - D));
  const float sin2t = 2.0f * c / D;
  const float cos2t = (a - b) / D;
  float ct, st;
  half_angle(sin2t, cos2t, &ct, &st);
  const float rs[4] = {s0 * ct, s0 * st, -s1 * st, s1 * ct};

  /* ndc (projection.comp:136-137) */
  float pc[4];
  mat4_vec4(cam->projection, pv, pc);
  const float nx = pc[0] / pc[3], ny = pc[1] / pc[3], nz = pc[2] / pc[3];

  /* SH degree 3 (projection.comp:140-174) */
  const float C0 = 0.28209479177387814f, C1 = 0.4886025119029199f, C20 = 1.0925484305920792f,
              C21 = 0.31539156525252005f, C22 = 0.5462742152960396f, C30 = 0.5900435899266435f,
              C31 = 2.890611442640554f, C32 = 0.4570457994644658f, C33 = 0.3731763325901154f,
              C34 = 1.445305721320277f;
  const float x = dir[0], y = dir[1], z = dir[2];
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  const float b0[4] = {C0, -C1 * y, C1 * z, -C1 * x};
  const float b1[4] = {C20 * xy, -C20 * yz, C21 * (2.0f * zz - xx - yy), -C20 * xz};
  const float b2[4] = {C22 * (xx - yy), -C30 * y * (3.0f * xx - yy), C31 * xy * z, -C32 * y * (4.0f * zz - xx - yy)};
  const float b3[4] = {C33 * z * (2.0f * zz - 3.0f * xx - 3.0f * yy), -C32 * x * (4.0f * zz - xx - yy),
                       C34 * z * (xx - yy), -C30 * x * (xx - 3.0f * yy)};
  const uint16_t* s = sh + 48 * (size_t)id;
  float color[3];
  for (int ch = 0; ch < 3; ++ch) {
    float g0[4], g1[4], g2[4], g3[4];
    for (int k = 0; k < 4; ++k) {
      g0[k] = or_f16_to_f32(s[ch * 16 + 0 + k]);
      g1[k] = or_f16_to_f32(s[ch * 16 + 4 + k]);
      g2[k] = or_f16_to_f32(s[ch * 16 + 8 + k]);
      g3[k] = or_f16_to_f32(s[ch * 16 + 12 + k]);
    }
    color[ch] = ((dot4f(b0, g0) + dot4f(b1, g1)) + dot4f(b2, g2)) + dot4f(b3, g3);
    color[ch] = fmaxf(color[ch] + 0.5f, 0.0f);
  }
  const float o = opacity[id];

  if (inst) {
    inst[0] = nx;
    inst[1] = ny;
    inst[2] = nz;
    inst[3] = 0.0f;
    inst[4] = rs[0];
    inst[5] = rs[1];
    inst[6] = rs[2];
    inst[7] = rs[3];
    inst[8] = color[0];
    inst[9] = color[1];
    inst[10] = color[2];
    inst[11] = o;
  }
  if (rec) {
    /* Raster record.  Drawn iff the quad is non-degenerate (s1 > 0 and a finite inverse
     * rot_scale; D = 0 or a negative s1^2 give NaN, which the rasteriser never draws) and the
     * fragment depth nz passes clipping (nz >= 0) and LESS against the cleared depth 1.0. */
    const float m00 = ct / s0, m01 = st / s0, m10 = -st / s1, m11 = ct / s1;
    const int drawn = (s1 > 0.0f) && isfinite(m00) && isfinite(m01) && isfinite(m10) && isfinite(m11) &&
                      (nz >= 0.0f) && (nz < 1.0f);
    rec[0] = nx;
    rec[1] = ny;
    rec[2] = m00;
    rec[3] = m01;
    rec[4] = m10;
    rec[5] = m11;
    rec[6] = nz;
    rec[7] = o;
    rec[8] = fminf(color[0], 1.0f);
    rec[9] = fminf(color[1], 1.0f);
    rec[10] = fminf(color[2], 1.0f);
    rec[11] = 0.0f;
    rec[12] = drawn ? 3.0f * (fabsf(rs[0]) + fabsf(rs[2])) : -1.0f;
    rec[13] = drawn ? 3.0f * (fabsf(rs[1]) + fabsf(rs[3])) : -1.0f;
    rec[14] = 0.0f;
    rec[15] = 0.0f;
  }
}

void or_project(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                const uint32_t* sorted_index, uint32_t v, const or_camera* cam, float* instance, float* record) {
  float cam_m[3];
  camera_model_position(cam, cam_m);
  const float lpx = 1.0f / (float)cam->width / (float)cam->width;
  const float lpy = 1.0f / (float)cam->height / (float)cam->height;
#pragma omp parallel for schedule(static)
  for (long long r = 0; r < (long long)v; ++r)
    project_one(position, cov3d, opacity, sh, sorted_index[r], cam, cam_m, lpx, lpy,
                instance ? instance + 12 * (size_t)r : NULL, record ? record + 16 * (size_t)r : NULL);
}

/* ------------------------------------------------------------------------- */
/* A7 + A8: splat.vert / splat.frag + fixed-function blend.                   */
/* ------------------------------------------------------------------------- */

static inline float q8(float x) {
  x = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
  return nearbyintf(x * 255.0f) / 255.0f;
}

/* Pixel range whose centres can lie inside [c - h, c + h] in NDC, padded by one pixel. */
static void pixel_range(float c, float h, uint32_t size, long* lo, long* hi) {
  const double a = ((double)c - (double)h + 1.0) * (double)size * 0.5 - 0.5;
  const double b = ((double)c + (double)h + 1.0) * (double)size * 0.5 - 0.5;
  double fa = floor(a) - 1.0, fb = ceil(b) + 1.0;
  if (fa < 0.0) fa = 0.0;
  if (fb > (double)size - 1.0) fb = (double)size - 1.0;
  *lo = (long)fa;
  *hi = (long)fb;
}

uint64_t or_raster(const float* record, uint32_t v, uint32_t width, uint32_t height, const float* depth_in,
                   int unorm8, float* image) {
  return or_raster_bands(record, v, width, height, depth_in, unorm8, 1, 0, image);
}

uint64_t or_raster_bands(const float* record, uint32_t v, uint32_t width, uint32_t height, const float* depth_in,
                         int unorm8, uint32_t band_stride, uint32_t band_offset, float* image) {
  const uint32_t band = 16;
  const long nbands = ((long)height + band - 1) / band;
  uint64_t total = 0;
  if (band_stride == 0) band_stride = 1;
  for (size_t i = 0; i < (size_t)width * height; ++i) {
    image[4 * i + 0] = 0.0f;
    image[4 * i + 1] = 0.0f;
    image[4 * i + 2] = 0.0f;
    image[4 * i + 3] = 1.0f;
  }
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
  for (long bi = 0; bi < nbands; ++bi) {
    if ((uint32_t)bi % band_stride != band_offset % band_stride) continue;
    const long y0 = bi * band, y1 = (y0 + band < (long)height) ? y0 + band : (long)height;
    uint64_t frag = 0;
    for (uint32_t r = 0; r < v; ++r) {
      const float* q = record + 16 * (size_t)r;
      if (!(q[12] >= 0.0f)) continue;
      long ylo, yhi, xlo, xhi;
      pixel_range(q[1], q[13], height, &ylo, &yhi);
      if (yhi < y0 || ylo >= y1) continue;
      if (ylo < y0) ylo = y0;
      if (yhi > y1 - 1) yhi = y1 - 1;
      pixel_range(q[0], q[12], width, &xlo, &xhi);
      const float cx = q[0], cy = q[1], m00 = q[2], m01 = q[3], m10 = q[4], m11 = q[5], cz = q[6], o = q[7];
      for (long py = ylo; py <= yhi; ++py) {
        const float ny = (float)(2 * py + 1) / (float)height - 1.0f;
        const float dy = ny - cy;
        for (long px = xlo; px <= xhi; ++px) {
          const float nx = (float)(2 * px + 1) / (float)width - 1.0f;
          const float dx = nx - cx;
          const float u = m00 * dx + m01 * dy;
          const float w = m10 * dx + m11 * dy;
          if (!(fabsf(u) <= 3.0f && fabsf(w) <= 3.0f)) continue;
          const size_t pix = (size_t)py * width + (size_t)px;
          if (depth_in && !(cz < depth_in[pix])) continue;
          ++frag;
          const float g = expf(-0.5f * (u * u + w * w));
          const float a = o * g;
          float* dst = image + 4 * pix;
          const float ia = 1.0f - a;
          if (unorm8) {
            dst[0] = q8(a * q[8] + ia * dst[0]);
            dst[1] = q8(a * q[9] + ia * dst[1]);
            dst[2] = q8(a * q[10] + ia * dst[2]);
            dst[3] = q8(a * a + ia * dst[3]);
          } else {
            dst[0] = a * q[8] + ia * dst[0];
            dst[1] = a * q[9] + ia * dst[1];
            dst[2] = a * q[10] + ia * dst[2];
            dst[3] = a * a + ia * dst[3];
          }
        }
      }
    }
    total += frag;
  }
  return total;
}

uint32_t or_render_frame(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                         uint32_t n, const or_camera* cam, const float* depth_in, int unorm8, uint32_t* key,
                         uint32_t* index, float* instance, float* image, uint64_t* fragments) {
  const uint32_t v = or_rank(position, n, cam, key, index);
  or_sort_kv(key, index, v);
  float* rec = (float*)malloc((size_t)(v ? v : 1) * 16 * sizeof(float));
  or_project(position, cov3d, opacity, sh, index, v, cam, instance, rec);
  const uint64_t f = or_raster(rec, v, cam->width, cam->height, depth_in, unorm8, image);
  if (fragments) *fragments = f;
  free(rec);
  return v;
}

/* ------------------------------------------------------------------------- */
/* FP64 twin: the same frame with the literal reference formulas in double.   */
/* ------------------------------------------------------------------------- */

typedef struct {
  double key;
  uint32_t id;
} kd_pair;

static int kd_cmp(const void* pa, const void* pb) {
  const kd_pair* a = (const kd_pair*)pa;
  const kd_pair* b = (const kd_pair*)pb;
  if (a->key < b->key) return -1;
  if (a->key > b->key) return 1;
  return (a->id < b->id) ? -1 : (a->id > b->id);
}

static void d_mat4_mul(const double a[16], const double b[16], double out[16]) {
  double r[16];
  for (int j = 0; j < 4; ++j)
    for (int i = 0; i < 4; ++i)
      M4(r, j, i) = M4(a, 0, i) * M4(b, j, 0) + M4(a, 1, i) * M4(b, j, 1) + M4(a, 2, i) * M4(b, j, 2) +
                    M4(a, 3, i) * M4(b, j, 3);
  memcpy(out, r, sizeof(r));
}

static void d_mat4_vec4(const double m[16], const double v[4], double out[4]) {
  for (int i = 0; i < 4; ++i)
    out[i] = M4(m, 0, i) * v[0] + M4(m, 1, i) * v[1] + M4(m, 2, i) * v[2] + M4(m, 3, i) * v[3];
}

static void d_mat3_mul(const double a[9], const double b[9], double out[9]) {
  double r[9];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i)
      M3(r, j, i) = M3(a, 0, i) * M3(b, j, 0) + M3(a, 1, i) * M3(b, j, 1) + M3(a, 2, i) * M3(b, j, 2);
  memcpy(out, r, sizeof(r));
}

static void d_sandwich(const double m4[16], double cov[9]) {
  double m[9], mt[9], t[9];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      M3(m, j, i) = M4(m4, j, i);
      M3(mt, i, j) = M4(m4, j, i);
    }
  d_mat3_mul(m, cov, t);
  d_mat3_mul(t, mt, cov);
}

uint32_t or_render_frame_f64(const float* position, const float* cov3d, const float* opacity, const uint16_t* sh,
                             uint32_t n, const or_camera* cam, double* image) {
  double P[16], V[16], Mm[16], PV[16], PVM[16];
  for (int i = 0; i < 16; ++i) {
    P[i] = cam->projection[i];
    V[i] = cam->view[i];
    Mm[i] = cam->model[i];
  }
  d_mat4_mul(P, V, PV);
  d_mat4_mul(PV, Mm, PVM);
  kd_pair* list = (kd_pair*)malloc((size_t)(n ? n : 1) * sizeof(kd_pair));
  uint32_t v = 0;
  for (uint32_t id = 0; id < n; ++id) {
    const double p[4] = {position[3 * (size_t)id], position[3 * (size_t)id + 1], position[3 * (size_t)id + 2], 1.0};
    double c[4];
    d_mat4_vec4(PVM, p, c);
    const double x = c[0] / c[3], y = c[1] / c[3], z = c[2] / c[3];
    if (fabs(x) <= 1.0 && fabs(y) <= 1.0 && z >= 0.0 && z <= 1.0) {
      list[v].key = 1.0 - z;
      list[v].id = id;
      ++v;
    }
  }
  qsort(list, v, sizeof(kd_pair), kd_cmp);

  float cam_mf[3];
  camera_model_position(cam, cam_mf);
  const double W = cam->width, H = cam->height;
  double* rec = (double*)malloc((size_t)(v ? v : 1) * 12 * sizeof(double));
#pragma omp parallel for schedule(static)
  for (long long r = 0; r < (long long)v; ++r) {
    const uint32_t id = list[r].id;
    const float* cv = cov3d + 6 * (size_t)id;
    double pos[4] = {position[3 * (size_t)id], position[3 * (size_t)id + 1], position[3 * (size_t)id + 2], 1.0};
    double d[3] = {pos[0] - cam_mf[0], pos[1] - cam_mf[1], pos[2] - cam_mf[2]};
    const double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double x = d[0] / dl, y = d[1] / dl, z = d[2] / dl;
    double cov[9] = {cv[0], cv[1], cv[2], cv[1], cv[3], cv[4], cv[2], cv[4], cv[5]};
    d_sandwich(Mm, cov);
    double p1[4], pv[4], pc[4];
    d_mat4_vec4(Mm, pos, p1);
    d_sandwich(V, cov);
    d_mat4_vec4(V, p1, pv);
    double J[9] = {-1.0 / pv[2], 0.0, 0.0, 0.0, -1.0 / pv[2], 0.0, pv[0] / (pv[2] * pv[2]), pv[1] / (pv[2] * pv[2]), 0.0};
    double Jt[9], t[9];
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) M3(Jt, j, i) = M3(J, i, j);
    d_mat3_mul(J, cov, t);
    d_mat3_mul(t, Jt, cov);
    const double p00 = M4(P, 0, 0), p01 = M4(P, 0, 1), p10 = M4(P, 1, 0), p11 = M4(P, 1, 1);
    const double c00 = M3(cov, 0, 0), c01 = M3(cov, 0, 1), c10 = M3(cov, 1, 0), c11 = M3(cov, 1, 1);
    /* (P2 * C2) * P2 in column-major 2x2 */
    const double t00 = p00 * c00 + p10 * c01, t01 = p01 * c00 + p11 * c01;
    const double t10 = p00 * c10 + p10 * c11, t11 = p01 * c10 + p11 * c11;
    double a = t00 * p00 + t10 * p01;
    double b = t01 * p10 + t11 * p11;
    const double c = t00 * p10 + t10 * p11;
    a += 1.0 / (W * W);
    b += 1.0 / (H * H);
    const double D = sqrt((a - b) * (a - b) + 4.0 * c * c);
    const double s0 = sqrt(0.5 * (a + b + D)), s1 = sqrt(0.5 * (a + b - D));
    const double th = atan2(2.0 * c / D, (a - b) / D) / 2.0;
    const double ct = cos(th), st = sin(th);
    d_mat4_vec4(P, pv, pc);
    const double nx = pc[0] / pc[3], ny = pc[1] / pc[3], nz = pc[2] / pc[3];
    const double C0 = 0.28209479177387814, C1 = 0.4886025119029199, C20 = 1.0925484305920792,
                 C21 = 0.31539156525252005, C22 = 0.5462742152960396, C30 = 0.5900435899266435,
                 C31 = 2.890611442640554, C32 = 0.4570457994644658, C33 = 0.3731763325901154,
                 C34 = 1.445305721320277;
    const double xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
    const double basis[16] = {C0,
                              -C1 * y,
                              C1 * z,
                              -C1 * x,
                              C20 * xy,
                              -C20 * yz,
                              C21 * (2.0 * zz - xx - yy),
                              -C20 * xz,
                              C22 * (xx - yy),
                              -C30 * y * (3.0 * xx - yy),
                              C31 * xy * z,
                              -C32 * y * (4.0 * zz - xx - yy),
                              C33 * z * (2.0 * zz - 3.0 * xx - 3.0 * yy),
                              -C32 * x * (4.0 * zz - xx - yy),
                              C34 * z * (xx - yy),
                              -C30 * x * (xx - 3.0 * yy)};
    double* q = rec + 12 * (size_t)r;
    for (int ch = 0; ch < 3; ++ch) {
      double acc = 0.0;
      for (int k = 0; k < 16; ++k) acc += basis[k] * (double)or_f16_to_f32(sh[48 * (size_t)id + ch * 16 + k]);
      acc += 0.5;
      if (acc < 0.0) acc = 0.0;
      if (acc > 1.0) acc = 1.0;
      q[8 + ch] = acc;
    }
    const int drawn = (s1 > 0.0) && (th == th) && (nz >= 0.0) && (nz < 1.0);
    q[0] = nx;
    q[1] = ny;
    q[2] = ct / s0;
    q[3] = st / s0;
    q[4] = -st / s1;
    q[5] = ct / s1;
    q[6] = drawn ? 3.0 * (fabs(s0 * ct) + fabs(s1 * st)) : -1.0;
    q[7] = drawn ? 3.0 * (fabs(s0 * st) + fabs(s1 * ct)) : -1.0;
    q[11] = opacity[id];
  }
  for (size_t i = 0; i < (size_t)cam->width * cam->height; ++i) {
    image[4 * i + 0] = 0.0;
    image[4 * i + 1] = 0.0;
    image[4 * i + 2] = 0.0;
    image[4 * i + 3] = 1.0;
  }
  const long nbands = ((long)cam->height + 15) / 16;
#pragma omp parallel for schedule(dynamic, 1)
  for (long bi = 0; bi < nbands; ++bi) {
    const long y0 = bi * 16, y1 = (y0 + 16 < (long)cam->height) ? y0 + 16 : (long)cam->height;
    for (uint32_t r = 0; r < v; ++r) {
      const double* q = rec + 12 * (size_t)r;
      if (!(q[6] >= 0.0)) continue;
      long ylo, yhi, xlo, xhi;
      pixel_range((float)q[1], (float)q[7], cam->height, &ylo, &yhi);
      if (yhi < y0 || ylo >= y1) continue;
      if (ylo < y0) ylo = y0;
      if (yhi > y1 - 1) yhi = y1 - 1;
      pixel_range((float)q[0], (float)q[6], cam->width, &xlo, &xhi);
      for (long py = ylo; py <= yhi; ++py) {
        const double dy = (2.0 * py + 1.0) / H - 1.0 - q[1];
        for (long px = xlo; px <= xhi; ++px) {
          const double dx = (2.0 * px + 1.0) / W - 1.0 - q[0];
          const double u = q[2] * dx + q[3] * dy, w = q[4] * dx + q[5] * dy;
          if (!(fabs(u) <= 3.0 && fabs(w) <= 3.0)) continue;
          const double a = q[11] * exp(-0.5 * (u * u + w * w));
          double* dst = image + 4 * ((size_t)py * cam->width + (size_t)px);
          dst[0] = a * q[8] + (1.0 - a) * dst[0];
          dst[1] = a * q[9] + (1.0 - a) * dst[1];
          dst[2] = a * q[10] + (1.0 - a) * dst[2];
          dst[3] = a * a + (1.0 - a) * dst[3];
        }
      }
    }
  }
  free(rec);
  free(list);
  return v;
}
