// glsl.hpp -- the subset of GLSL 4.60 that the reference's splat shaders use, as C++17, so that the
// shader bodies (src/shader/{parse_ply,rank,inverse_index,projection}.comp, splat.vert, splat.frag)
// compile and run on the host without a graphics stack.
//
// TEST INFRASTRUCTURE ONLY: the executable reference that pins the oracle (oracle/cpu_ref.c).  Nothing
// in the product links it.
//
// Arithmetic model (the one thing GLSL leaves to the implementation, fixed here and stated so the pin
// can be read): every +, -, *, / and sqrt is one IEEE binary32 rounding (build with
// -ffp-contract=off, no -ffast-math); exp/atan/cos/sin are the C library's expf/atan2f/cosf/sinf;
// dot products and matrix products sum their terms left to right (k = 0, 1, 2, ...);
// normalize(v) = v / length(v), length(v) = sqrt(dot(v, v)); float16_t(x) rounds to nearest even.
// Matrices are column-major: m[c] is column c, m[c][r] the element in row r, constructors fill
// columns first, as GLSL does.
#pragma once

#include <cstdint>
#include <cstring>

extern "C" {
float sqrtf(float);
float expf(float);
float atan2f(float, float);
float cosf(float);
float sinf(float);
float fabsf(float);
}

namespace glsl {

using uint = uint32_t;

struct vec2;
struct vec3;
struct vec4;
struct float16_t;
struct f16vec4;

// ---- component lists for the constructors: scalars, vectors and swizzles flatten in order --------
struct comps {
  float v[16];
  int n = 0;
};
inline void push(comps& c, float x) { c.v[c.n++] = x; }
inline void push(comps& c, double x) { c.v[c.n++] = (float)x; }
inline void push(comps& c, int x) { c.v[c.n++] = (float)x; }
inline void push(comps& c, uint x) { c.v[c.n++] = (float)x; }
inline void push(comps& c, const vec2& x);
inline void push(comps& c, const vec3& x);
inline void push(comps& c, const vec4& x);
inline void push(comps& c, const float16_t& x);
inline void push(comps& c, const f16vec4& x);

// A swizzle of N-component storage selecting components I... (read as V, assignable from V).
template <class V, int N, int... I>
struct swz {
  float e[N];
  operator V() const { return V(e[I]...); }
  swz& operator=(const V& v) {
    int k = 0;
    ((e[I] = v.e[k++]), ...);
    return *this;
  }
  swz& operator=(const swz& o) { return *this = V(o); }
};
template <class V, int N, int... I>
inline void push(comps& c, const swz<V, N, I...>& s) {
  (push(c, s.e[I]), ...);
}

#define GLSL_VEC_COMMON(T, N)                                        \
  T() { std::memset(e, 0, sizeof e); }                               \
  T(const T& o) { std::memcpy(e, o.e, sizeof e); }                   \
  T& operator=(const T& o) {                                         \
    std::memcpy(e, o.e, sizeof e);                                   \
    return *this;                                                    \
  }                                                                  \
  template <class... A>                                              \
  explicit T(const A&... a) {                                        \
    comps c;                                                         \
    (push(c, a), ...);                                               \
    for (int i = 0; i < N; ++i) e[i] = c.n == 1 ? c.v[0] : c.v[i];  \
  }                                                                  \
  float& operator[](int i) { return e[i]; }                          \
  float operator[](int i) const { return e[i]; }

struct vec2 {
  union {
    float e[2];
    struct {
      float x, y;
    };
    struct {
      float r, g;
    };
  };
  GLSL_VEC_COMMON(vec2, 2)
};

struct vec3 {
  union {
    float e[3];
    struct {
      float x, y, z;
    };
    struct {
      float r, g, b;
    };
    swz<vec2, 3, 0, 1> xy;
    swz<vec2, 3, 1, 2> yz;
    swz<vec2, 3, 0, 2> xz;
  };
  GLSL_VEC_COMMON(vec3, 3)
};

struct vec4 {
  union {
    float e[4];
    struct {
      float x, y, z, w;
    };
    struct {
      float r, g, b, a;
    };
    swz<vec2, 4, 0, 1> xy;
    swz<vec2, 4, 1, 2> yz;
    swz<vec2, 4, 2, 3> zw;
    swz<vec3, 4, 0, 1, 2> xyz;
    swz<vec3, 4, 0, 1, 2> rgb;
  };
  GLSL_VEC_COMMON(vec4, 4)
};
#undef GLSL_VEC_COMMON

struct uvec2 {
  uint x = 0, y = 0;
};
struct uvec3 {
  uint x = 0, y = 0, z = 0;
};

inline void push(comps& c, const vec2& x) {
  for (float f : x.e) push(c, f);
}
inline void push(comps& c, const vec3& x) {
  for (float f : x.e) push(c, f);
}
inline void push(comps& c, const vec4& x) {
  for (float f : x.e) push(c, f);
}

// ---- binary16 storage (GL_EXT_shader_16bit_storage) ------------------------------------------------
struct float16_t {
  uint16_t bits;
  float16_t() = default;
  explicit float16_t(float f) : bits(from_float(f)) {}
  operator float() const { return to_float(bits); }

  static uint16_t from_float(float f) {  // round to nearest, ties to even; overflow -> inf; NaN kept
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t sign = (u >> 16) & 0x8000u;
    const uint32_t ex = (u >> 23) & 0xffu;
    uint32_t man = u & 0x7fffffu;
    if (ex == 0xffu) return (uint16_t)(sign | 0x7c00u | (man ? 0x200u : 0u));
    const int e = (int)ex - 127 + 15;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {  // subnormal half (or zero)
      if (e < -10) return (uint16_t)sign;
      man |= 0x800000u;
      const int shift = 14 - e;  // 24-bit significand -> 10 - (1 - e) bits
      const uint32_t half = man >> shift, rem = man & ((1u << shift) - 1u), mid = 1u << (shift - 1);
      const uint32_t r = half + ((rem > mid || (rem == mid && (half & 1u))) ? 1u : 0u);
      return (uint16_t)(sign | r);
    }
    const uint32_t half = ((uint32_t)e << 10) | (man >> 13), rem = man & 0x1fffu;
    const uint32_t r = half + ((rem > 0x1000u || (rem == 0x1000u && (half & 1u))) ? 1u : 0u);
    return (uint16_t)(sign | r);  // a carry into the exponent (up to inf) is the correct rounding
  }
  static float to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t ex = (h >> 10) & 0x1fu, man = h & 0x3ffu, u;
    if (ex == 0x1fu) {
      u = sign | 0x7f800000u | (man << 13);
    } else if (ex == 0) {
      if (man == 0) {
        u = sign;
      } else {  // subnormal: normalise
        int e = -1;
        do {
          ++e;
          man <<= 1;
        } while (!(man & 0x400u));
        u = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3ffu) << 13);
      }
    } else {
      u = sign | ((ex + 127 - 15) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &u, 4);
    return f;
  }
};
static_assert(sizeof(float16_t) == 2, "binary16 storage");

struct f16vec4 {
  float16_t x, y, z, w;
};
static_assert(sizeof(f16vec4) == 8, "f16vec4 storage");
inline void push(comps& c, const float16_t& x) { push(c, (float)x); }
inline void push(comps& c, const f16vec4& x) {
  push(c, (float)x.x);
  push(c, (float)x.y);
  push(c, (float)x.z);
  push(c, (float)x.w);
}

// ---- matrices (column-major) -------------------------------------------------------------------------
template <class Col, int C>
struct matc {
  Col c[C];
  Col& operator[](int i) { return c[i]; }
  const Col& operator[](int i) const { return c[i]; }
};

struct mat4;
struct mat3;

struct mat2 : matc<vec2, 2> {
  mat2() = default;
  template <class... A>
  explicit mat2(const A&... a) {
    comps cs;
    (push(cs, a), ...);
    fill(cs);
  }
  explicit mat2(const mat3& m);
  explicit mat2(const mat4& m);
  void fill(const comps& cs) {
    if (cs.n == 1) {
      c[0] = vec2(cs.v[0], 0.0f);
      c[1] = vec2(0.0f, cs.v[0]);
      return;
    }
    for (int i = 0; i < 4; ++i) c[i / 2][i % 2] = cs.v[i];
  }
};

struct mat3 : matc<vec3, 3> {
  mat3() = default;
  template <class... A>
  explicit mat3(const A&... a) {
    comps cs;
    (push(cs, a), ...);
    if (cs.n == 1) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) c[i][j] = i == j ? cs.v[0] : 0.0f;
      return;
    }
    for (int i = 0; i < 9; ++i) c[i / 3][i % 3] = cs.v[i];
  }
  explicit mat3(const mat4& m);
};

struct mat4 : matc<vec4, 4> {
  mat4() = default;
  template <class... A>
  explicit mat4(const A&... a) {
    comps cs;
    (push(cs, a), ...);
    if (cs.n == 1) {
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) c[i][j] = i == j ? cs.v[0] : 0.0f;
      return;
    }
    for (int i = 0; i < 16; ++i) c[i / 4][i % 4] = cs.v[i];
  }
};

// mat3x4: three columns of four rows
struct mat3x4 : matc<vec4, 3> {
  mat3x4() = default;
  template <class... A>
  explicit mat3x4(const A&... a) {
    comps cs;
    (push(cs, a), ...);
    for (int i = 0; i < 12; ++i) c[i / 4][i % 4] = cs.v[i];
  }
};

inline mat2::mat2(const mat3& m) {
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) c[i][j] = m[i][j];
}
inline mat2::mat2(const mat4& m) {
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) c[i][j] = m[i][j];
}
inline mat3::mat3(const mat4& m) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c[i][j] = m[i][j];
}

// ---- vector arithmetic (component-wise) --------------------------------------------------------------
#define GLSL_VEC_OPS(T, N)                                                      \
  inline T operator+(const T& a, const T& b) {                                  \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] + b.e[i];                       \
    return r;                                                                   \
  }                                                                             \
  inline T operator-(const T& a, const T& b) {                                  \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] - b.e[i];                       \
    return r;                                                                   \
  }                                                                             \
  inline T operator*(const T& a, const T& b) {                                  \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] * b.e[i];                       \
    return r;                                                                   \
  }                                                                             \
  inline T operator/(const T& a, const T& b) {                                  \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] / b.e[i];                       \
    return r;                                                                   \
  }                                                                             \
  inline T operator+(const T& a, float s) {                                     \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] + s;                            \
    return r;                                                                   \
  }                                                                             \
  inline T operator-(const T& a, float s) {                                     \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] - s;                            \
    return r;                                                                   \
  }                                                                             \
  inline T operator*(const T& a, float s) {                                     \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] * s;                            \
    return r;                                                                   \
  }                                                                             \
  inline T operator*(float s, const T& a) {                                     \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = s * a.e[i];                            \
    return r;                                                                   \
  }                                                                             \
  inline T operator/(const T& a, float s) {                                     \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] / s;                            \
    return r;                                                                   \
  }                                                                             \
  inline T operator-(const T& a) {                                              \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = -a.e[i];                               \
    return r;                                                                   \
  }                                                                             \
  inline T& operator+=(T& a, const T& b) { return a = a + b; }                  \
  inline float dot(const T& a, const T& b) {                                    \
    float s = a.e[0] * b.e[0];                                                  \
    for (int i = 1; i < N; ++i) s = s + a.e[i] * b.e[i];                        \
    return s;                                                                   \
  }                                                                             \
  inline float length(const T& a) { return sqrtf(dot(a, a)); }                  \
  inline T normalize(const T& a) { return a / length(a); }                      \
  inline T max(const T& a, float s) {                                           \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = a.e[i] < s ? s : a.e[i];               \
    return r;                                                                   \
  }                                                                             \
  inline T exp(const T& a) {                                                    \
    T r;                                                                        \
    for (int i = 0; i < N; ++i) r.e[i] = expf(a.e[i]);                          \
    return r;                                                                   \
  }
GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)
#undef GLSL_VEC_OPS

// ---- matrix products: element (row r, column c) = sum_k a[k][r] * b[c][k], k ascending ---------------
template <class M, class Col, int C>
inline M matmul(const M& a, const M& b) {
  M out;
  for (int c = 0; c < C; ++c)
    for (int r = 0; r < C; ++r) {
      float s = a[0][r] * b[c][0];
      for (int k = 1; k < C; ++k) s = s + a[k][r] * b[c][k];
      out[c][r] = s;
    }
  return out;
}
inline mat2 operator*(const mat2& a, const mat2& b) { return matmul<mat2, vec2, 2>(a, b); }
inline mat3 operator*(const mat3& a, const mat3& b) { return matmul<mat3, vec3, 3>(a, b); }
inline mat4 operator*(const mat4& a, const mat4& b) { return matmul<mat4, vec4, 4>(a, b); }

template <class M, class V, int C, int R>
inline V matvec(const M& m, const V& v) {  // column vector: r[i] = sum_k m[k][i] v[k]
  V out;
  for (int i = 0; i < R; ++i) {
    float s = m[0][i] * v.e[0];
    for (int k = 1; k < C; ++k) s = s + m[k][i] * v.e[k];
    out.e[i] = s;
  }
  return out;
}
inline vec2 operator*(const mat2& m, const vec2& v) { return matvec<mat2, vec2, 2, 2>(m, v); }
inline vec3 operator*(const mat3& m, const vec3& v) { return matvec<mat3, vec3, 3, 3>(m, v); }
inline vec4 operator*(const mat4& m, const vec4& v) { return matvec<mat4, vec4, 4, 4>(m, v); }

// row vector times matrix: r[j] = dot(v, m[j]) (OpVectorTimesMatrix)
inline vec3 operator*(const vec4& v, const mat3x4& m) { return vec3(dot(v, m[0]), dot(v, m[1]), dot(v, m[2])); }

inline mat3 transpose(const mat3& m) {
  mat3 t;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[i][j] = m[j][i];
  return t;
}
inline mat2 transpose(const mat2& m) {
  mat2 t;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) t[i][j] = m[j][i];
  return t;
}

// inverse(mat4): adjugate over the determinant (Laplace expansion by 2x2 minors), in binary32.
inline mat4 inverse(const mat4& m) {
  auto a = [&](int c, int r) { return m[c][r]; };
  const float s0 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1), s1 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
  const float s2 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3), s3 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
  const float s4 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3), s5 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
  const float c5 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3), c4 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
  const float c3 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2), c2 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
  const float c1 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2), c0 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
  const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
  const float id = 1.0f / det;
  // rows of the adjugate indexed (row, column) of the inverse
  float inv[4][4];
  inv[0][0] = (a(1, 1) * c5 - a(1, 2) * c4 + a(1, 3) * c3) * id;
  inv[0][1] = (-a(0, 1) * c5 + a(0, 2) * c4 - a(0, 3) * c3) * id;
  inv[0][2] = (a(3, 1) * s5 - a(3, 2) * s4 + a(3, 3) * s3) * id;
  inv[0][3] = (-a(2, 1) * s5 + a(2, 2) * s4 - a(2, 3) * s3) * id;
  inv[1][0] = (-a(1, 0) * c5 + a(1, 2) * c2 - a(1, 3) * c1) * id;
  inv[1][1] = (a(0, 0) * c5 - a(0, 2) * c2 + a(0, 3) * c1) * id;
  inv[1][2] = (-a(3, 0) * s5 + a(3, 2) * s2 - a(3, 3) * s1) * id;
  inv[1][3] = (a(2, 0) * s5 - a(2, 2) * s2 + a(2, 3) * s1) * id;
  inv[2][0] = (a(1, 0) * c4 - a(1, 1) * c2 + a(1, 3) * c0) * id;
  inv[2][1] = (-a(0, 0) * c4 + a(0, 1) * c2 - a(0, 3) * c0) * id;
  inv[2][2] = (a(3, 0) * s4 - a(3, 1) * s2 + a(3, 3) * s0) * id;
  inv[2][3] = (-a(2, 0) * s4 + a(2, 1) * s2 - a(2, 3) * s0) * id;
  inv[3][0] = (-a(1, 0) * c3 + a(1, 1) * c1 - a(1, 2) * c0) * id;
  inv[3][1] = (a(0, 0) * c3 - a(0, 1) * c1 + a(0, 2) * c0) * id;
  inv[3][2] = (-a(3, 0) * s3 + a(3, 1) * s1 - a(3, 2) * s0) * id;
  inv[3][3] = (a(2, 0) * s3 - a(2, 1) * s1 + a(2, 2) * s0) * id;
  mat4 out;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) out[c][r] = inv[c][r];
  return out;
}

// ---- scalar built-ins ----------------------------------------------------------------------------------
inline float abs(float x) { return fabsf(x); }
inline float max(float a, float b) { return a < b ? b : a; }
inline float sqrt(float x) { return sqrtf(x); }
inline float exp(float x) { return expf(x); }
inline float atan(float y, float x) { return atan2f(y, x); }
inline float cos(float x) { return cosf(x); }
inline float sin(float x) { return sinf(x); }
inline uint floatBitsToUint(float x) {
  uint u;
  std::memcpy(&u, &x, 4);
  return u;
}
// Invocations run one at a time, so the atomic is a plain fetch-and-add in invocation order.
inline uint atomicAdd(uint& mem, uint v) {
  const uint old = mem;
  mem = old + v;
  return old;
}
inline uint atomicAdd(uint& mem, int v) { return atomicAdd(mem, (uint)v); }
// The harness runs the part of a workgroup before a barrier for every invocation first.
inline void barrier() {}

}  // namespace glsl
