// ORACLE — test infrastructure only.  The GLSL language pieces the
// reference's compute shaders use, in C++, so that their own function
// bodies (transliterated by oracle/build_ref.py, which rewrites only what
// C++ cannot parse) compile and run on the CPU.  Included INSIDE one
// namespace per shader, after <cmath>, <cstdint> and <cstring> at global
// scope: unqualified calls in the shader (log, max, pow ...) then find the
// float versions declared here before any C library overload.
//
// Semantics follow the GLSL 4.50 specification: vectors are componentwise,
// a scalar operand of any arithmetic type converts to float, mix(x, y, a) =
// x (1 - a) + y a, smoothstep(e0, e1, x) = t^2 (3 - 2 t) with t clamped
// (x - e0) / (e1 - e0), matrices are column-major (m * v sums the columns
// weighted by v's components), a global variable is private to its
// invocation (the transliteration declares it thread_local).  Arithmetic is
// IEEE float32 with no contraction (-ffp-contract=off); the functions are
// the C library's.
//
// texture() is the sampler the reference binds (Initializers.cpp:408-418):
// linear filtering and clamp-to-edge on all axes, written from Vulkan's
// linear-filter formula (u = s N - 1/2, texels floor(u) and floor(u) + 1
// clamped to [0, N - 1], weights 1 - frac(u) and frac(u)) in float32; an
// R32F texture reads as (r, 0, 0, 1).

using uint = uint32_t;

struct vec2 {
  float x, y;
  vec2() = default;
  constexpr vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
  float x, y, z;
  vec3() = default;
  constexpr explicit vec3(float s) : x(s), y(s), z(s) {}
  constexpr vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  float& operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
};

struct vec4 {
  union {
    struct {
      float x, y, z, w;
    };
    vec3 xyz;
  };
  vec4() : x(0), y(0), z(0), w(0) {}
  constexpr explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
  constexpr vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
  vec4& operator=(const vec4& o) {
    x = o.x; y = o.y; z = o.z; w = o.w;
    return *this;
  }
  float& operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
};

struct uvec2 {
  uint x, y;
};
struct ivec2 {
  int x, y;
  ivec2() = default;
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(const uvec2& u) : x((int)u.x), y((int)u.y) {}
};
struct uvec3 {
  union {
    struct {
      uint x, y, z;
    };
    uvec2 xy;
  };
  uvec3() : x(0), y(0), z(0) {}
  uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
  uvec3(const uvec2& v, uint c) : x(v.x), y(v.y), z(c) {}
};
struct ivec3 {
  int x, y, z;
  ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
  ivec3(const uvec2& v, uint c) : x((int)v.x), y((int)v.y), z((int)c) {}
};
struct uvec4 {
  uint x, y, z, w;
};

struct mat4 {
  vec4 c[4];  // columns
};

// ---- vector arithmetic ------------------------------------------------------
template <class S>
using if_scalar = typename std::enable_if<std::is_arithmetic<S>::value, int>::type;

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
template <class S, if_scalar<S> = 0>
inline vec3 operator*(const vec3& a, S s) { const float f = (float)s; return vec3(a.x * f, a.y * f, a.z * f); }
template <class S, if_scalar<S> = 0>
inline vec3 operator*(S s, const vec3& a) { const float f = (float)s; return vec3(f * a.x, f * a.y, f * a.z); }
template <class S, if_scalar<S> = 0>
inline vec3 operator/(S s, const vec3& a) { const float f = (float)s; return vec3(f / a.x, f / a.y, f / a.z); }
template <class S, if_scalar<S> = 0>
inline vec3 operator/(const vec3& a, S s) { const float f = (float)s; return vec3(a.x / f, a.y / f, a.z / f); }

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const vec4& a, const vec4& b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4 operator/(const vec4& a, const vec4& b) { return vec4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
inline vec4 operator-(const vec4& a) { return vec4(-a.x, -a.y, -a.z, -a.w); }
template <class S, if_scalar<S> = 0>
inline vec4 operator*(const vec4& a, S s) {
  const float f = (float)s;
  return vec4(a.x * f, a.y * f, a.z * f, a.w * f);
}
template <class S, if_scalar<S> = 0>
inline vec4 operator*(S s, const vec4& a) {
  const float f = (float)s;
  return vec4(f * a.x, f * a.y, f * a.z, f * a.w);
}
template <class S, if_scalar<S> = 0>
inline vec4 operator/(const vec4& a, S s) {
  const float f = (float)s;
  return vec4(a.x / f, a.y / f, a.z / f, a.w / f);
}
inline vec4& operator+=(vec4& a, const vec4& b) { return a = a + b; }
template <class S, if_scalar<S> = 0>
inline vec4& operator/=(vec4& a, S s) { return a = a / s; }

// column-major: m * v = c0 v.x + c1 v.y + c2 v.z + c3 v.w
inline vec4 operator*(const mat4& m, const vec4& v) {
  vec4 r;
  for (int i = 0; i < 4; ++i)
    r[i] = ((m.c[0][i] * v.x + m.c[1][i] * v.y) + m.c[2][i] * v.z) + m.c[3][i] * v.w;
  return r;
}

// ---- built-in functions -------------------------------------------------------
inline float abs(float x) { return std::fabs(x); }
inline float max(float a, float b) { return a < b ? b : a; }
inline float min(float a, float b) { return b < a ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float acos(float x) { return std::acos(x); }
inline float atan(float y, float x) { return std::atan2(y, x); }
inline float log(float x) { return std::log(x); }
inline float exp(float x) { return std::exp(x); }
inline vec4 exp(const vec4& v) { return vec4(exp(v.x), exp(v.y), exp(v.z), exp(v.w)); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& a) { return sqrt(dot(a, a)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec3 normalize(const vec3& a) { return a / length(a); }
inline float smoothstep(float e0, float e1, float x) {
  const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
inline vec4 mix(const vec4& a, const vec4& b, float t) { return a * (1.0f - t) + b * t; }

// ---- resources ------------------------------------------------------------------
struct sampler3D {
  const float* texels = nullptr;  // x fastest
  int n[3] = {0, 0, 0};
};

inline vec4 texture(const sampler3D& s, const vec3& p) {
  int i0[3], i1[3];
  float a[3];
  for (int k = 0; k < 3; ++k) {
    const float u = p[k] * (float)s.n[k] - 0.5f;
    const float f = std::floor(u);
    a[k] = u - f;
    const int lo = (int)f;
    i0[k] = lo < 0 ? 0 : (lo > s.n[k] - 1 ? s.n[k] - 1 : lo);
    i1[k] = lo + 1 < 0 ? 0 : (lo + 1 > s.n[k] - 1 ? s.n[k] - 1 : lo + 1);
  }
  auto at = [&](int x, int y, int z) { return s.texels[(size_t)x + (size_t)s.n[0] * ((size_t)y + (size_t)s.n[1] * z)]; };
  const float c00 = at(i0[0], i0[1], i0[2]) * (1.0f - a[0]) + at(i1[0], i0[1], i0[2]) * a[0];
  const float c10 = at(i0[0], i1[1], i0[2]) * (1.0f - a[0]) + at(i1[0], i1[1], i0[2]) * a[0];
  const float c01 = at(i0[0], i0[1], i1[2]) * (1.0f - a[0]) + at(i1[0], i0[1], i1[2]) * a[0];
  const float c11 = at(i0[0], i1[1], i1[2]) * (1.0f - a[0]) + at(i1[0], i1[1], i1[2]) * a[0];
  const float c0 = c00 * (1.0f - a[1]) + c10 * a[1];
  const float c1 = c01 * (1.0f - a[1]) + c11 * a[1];
  return vec4(c0 * (1.0f - a[2]) + c1 * a[2], 0.0f, 0.0f, 1.0f);
}

struct image2D {
  float* rgba = nullptr;  // width x height x 4, row-major
  int width = 0;
};
inline vec4 imageLoad(const image2D& im, const ivec2& p) {
  const float* q = im.rgba + 4 * ((size_t)p.y * im.width + p.x);
  return vec4(q[0], q[1], q[2], q[3]);
}
inline void imageStore(image2D& im, const ivec2& p, const vec4& v) {
  float* q = im.rgba + 4 * ((size_t)p.y * im.width + p.x);
  q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w;
}

struct image3D {
  float* r = nullptr;  // n x n x n, x fastest (R32F)
  int n = 0;
};
inline void imageStore(image3D& im, const ivec3& p, const vec4& v) {
  im.r[(size_t)p.x + (size_t)im.n * ((size_t)p.y + (size_t)im.n * p.z)] = v.x;
}

// ---- the built-in inputs of a compute invocation (per invocation) -------------
inline thread_local uvec3 gl_GlobalInvocationID;
inline uvec3 gl_WorkGroupSize(32, 32, 1);
inline uvec3 gl_NumWorkGroups(1, 1, 1);

// ---- the uniform blocks (the reference's declarations, by name and member) ----
struct CameraPropertiesBlock {
  vec3 position;
  int halfWidth;
  vec3 forward;
  int halfHeight;
  vec3 right;
  float nearPlane;
  vec3 up;
  float pixelSizeY;
  float pixelSizeX;
};
struct CloudPropertiesBlock {
  vec4 bounds[2];
  uvec4 voxelCount;
  float maxExtinction;
  float baseScaling;
  float densityScaling;
};
struct ParametersBlock {
  uint maxRayBounces;
  float lightIntensity;
  float phaseG;
  float phaseOnePlusG2;
  float phaseOneMinusG2;
  float phaseOneOver2G;
  bool isotropic;
};
struct ShadowVolumePropertiesBlock {
  vec4 bounds[2];
  vec4 lightDirection;
  vec4 right;
  vec4 up;
  mat4 basisChange;
  uint voxelAxisCount;
  float voxelSize;
};
struct PushConstantsBlock {
  double time;
  int seed;
  uint frameCount;
  float pmRadius;
};
