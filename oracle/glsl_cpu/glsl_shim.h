/* Oracle (test infrastructure only): a minimal GLSL-compute emulation layer that
 * lets the reference's own shader files (shaders/sph_common.glsl plus one pass
 * body) compile unmodified as C++ and run on the CPU.
 *
 * This header is included INSIDE a per-pass namespace (see glsl_passes.cpp), so
 * every pass gets private copies of the push-constant block, the image
 * bindings and gl_GlobalInvocationID, exactly like one compiled shader
 * program. It deliberately includes no standard header: the GLSL builtins
 * below (pow, floor, sqrt, min, max, clamp, ...) must be the only candidates
 * that unqualified calls in the shader source can find.
 *
 * Semantics mirrored from GLSL 4.x:
 *  - vecN / ivecN value types with .x .y .z .w (.r alias) and a read-only
 *    .xyz swizzle (the only multi-component swizzle the shaders use);
 *  - scalar/vector arithmetic, component-wise comparisons, all();
 *  - imageLoad / imageStore over RGBA32F or R32F 2-D images addressed by texel
 *    (flat arrays wrapped at a fixed width, as solver/gpu_util.py:28-30 lays
 *    them out) and one R32F 3-D image; out-of-range loads return 0 and
 *    out-of-range stores are dropped, as GLSL image access does;
 *  - floatBitsToInt / intBitsToFloat bit casts.
 * Unsuffixed literals such as 0.4 are double in C++ and float in GLSL: the
 * harness is compiled with -fsingle-precision-constant (and -ffp-contract=off),
 * so they are float here too and every expression rounds as the shader
 * writes it. pow() is glibc's powf, correctly rounded; GLSL leaves pow's
 * precision to the implementation (it inherits exp2(y * log2(x))'s), so an
 * integer power such as sph_delta.glsl's pow(ratio, 4.0) may differ by an
 * ulp from a restatement that squares twice.
 */

/* ---- scalar builtins -------------------------------------------------- */
inline float pow(float a, float b) { return __builtin_powf(a, b); }
inline float sqrt(float a) { return __builtin_sqrtf(a); }
inline float floor(float a) { return __builtin_floorf(a); }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline int floatBitsToInt(float f)
{
  int i;
  __builtin_memcpy(&i, &f, sizeof i);
  return i;
}
inline float intBitsToFloat(int i)
{
  float f;
  __builtin_memcpy(&f, &i, sizeof f);
  return f;
}

/* ---- vector types ----------------------------------------------------- */
struct ivec3;

struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3(const ivec3 &v);
  vec3 &operator+=(const vec3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
  vec3 &operator-=(const vec3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  vec3 &operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
};

struct ivec3 {
  int x, y, z;
  ivec3() : x(0), y(0), z(0) {}
  ivec3(int s) : x(s), y(s), z(s) {}
  ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
  explicit ivec3(const vec3 &v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
};
inline vec3::vec3(const ivec3 &v) : x((float)v.x), y((float)v.y), z((float)v.z) {}

struct ivec2 {
  int x, y;
  ivec2(int a, int b) : x(a), y(b) {}
};

struct uvec3 {
  unsigned x, y, z;
};

struct bvec3 {
  bool x, y, z;
};

/* Read-only .xyz swizzle overlaid on a 4-component vector's storage. */
struct swz3f {
  float v[4];
  operator vec3() const { return vec3(v[0], v[1], v[2]); }
};
struct swz3i {
  int v[4];
  operator ivec3() const { return ivec3(v[0], v[1], v[2]); }
};

struct vec4 {
  union {
    struct { float x, y, z, w; };
    struct { float r, g, b, a; };
    swz3f xyz;
  };
  vec4() : x(0), y(0), z(0), w(0) {}
  vec4(float s) : x(s), y(s), z(s), w(s) {}
  vec4(float a_, float b_, float c_, float d_) : x(a_), y(b_), z(c_), w(d_) {}
  vec4(const vec3 &v, float d_) : x(v.x), y(v.y), z(v.z), w(d_) {}
};

struct ivec4 {
  union {
    struct { int x, y, z, w; };
    swz3i xyz;
  };
  ivec4() : x(0), y(0), z(0), w(0) {}
};

/* ---- vector arithmetic ------------------------------------------------ */
inline vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator+(const vec3 &a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator*(const vec3 &a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3 &a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3 &a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator-(const vec3 &a) { return vec3(-a.x, -a.y, -a.z); }

inline ivec3 operator+(const ivec3 &a, const ivec3 &b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(const ivec3 &a, int s) { return ivec3(a.x - s, a.y - s, a.z - s); }

inline float dot(const vec3 &a, const vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(const vec3 &a) { return sqrt(dot(a, a)); }
inline vec3 floor(const vec3 &a) { return vec3(floor(a.x), floor(a.y), floor(a.z)); }
inline ivec3 clamp(const ivec3 &x, const ivec3 &lo, const ivec3 &hi)
{
  return ivec3(clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y), clamp(x.z, lo.z, hi.z));
}
inline bvec3 greaterThanEqual(const ivec3 &a, const ivec3 &b)
{
  return bvec3{a.x >= b.x, a.y >= b.y, a.z >= b.z};
}
inline bvec3 lessThan(const ivec3 &a, const ivec3 &b)
{
  return bvec3{a.x < b.x, a.y < b.y, a.z < b.z};
}
inline bool all(const bvec3 &b) { return b.x && b.y && b.z; }

/* ---- images ------------------------------------------------------------ */
struct image2D {
  float *data;
  int width, height, channels;
};
struct image3D {
  float *data;
  int dx, dy, dz;
};

inline vec4 imageLoad(const image2D &img, ivec2 t)
{
  if (!img.data || t.x < 0 || t.y < 0 || t.x >= img.width || t.y >= img.height) {
    return vec4(0.0f);
  }
  const float *p = img.data + ((long)t.y * img.width + t.x) * img.channels;
  if (img.channels == 4) {
    return vec4(p[0], p[1], p[2], p[3]);
  }
  return vec4(p[0], 0.0f, 0.0f, 1.0f);
}

inline void imageStore(const image2D &img, ivec2 t, const vec4 &v)
{
  if (!img.data || t.x < 0 || t.y < 0 || t.x >= img.width || t.y >= img.height) {
    return;
  }
  float *p = img.data + ((long)t.y * img.width + t.x) * img.channels;
  p[0] = v.x;
  if (img.channels == 4) {
    p[1] = v.y;
    p[2] = v.z;
    p[3] = v.w;
  }
}

inline vec4 imageLoad(const image3D &img, const ivec3 &c)
{
  if (!img.data || c.x < 0 || c.y < 0 || c.z < 0 || c.x >= img.dx || c.y >= img.dy ||
      c.z >= img.dz) {
    return vec4(0.0f);
  }
  return vec4(img.data[((long)c.z * img.dy + c.y) * img.dx + c.x], 0.0f, 0.0f, 1.0f);
}
