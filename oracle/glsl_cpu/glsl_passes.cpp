/* Oracle (test infrastructure only): the reference's PBF compute passes, built
 * from its own GLSL sources, unmodified, for the CPU.
 *
 * Each pass is compiled into its own namespace from
 *   glsl_shim.h + shaders/sph_common.glsl + shaders/<pass>.glsl
 * which is the same concatenation solver/sph.py:395-405 (_compile_passes) and
 * solver/surface.py:143-152 (start) hand to Blender's shader compiler. The
 * shader directory is passed on the compiler command line (-I), so no shader
 * text is copied into this repository. Invocations of one dispatch run in
 * parallel with OpenMP; every reference pass writes only texels it owns
 * (sph_cell_range.glsl:4-7, sph_sort.glsl:10-11), so this is race-free.
 *
 * Built by oracle/glsl_cpu/Makefile into oracle/_ref/libglslref.so. It needs the
 * reference sources, so it exists only where they are mounted; the parity
 * fixtures under tests/golden/ are generated from it.
 */
#include <stdint.h>

extern "C" {
/* The 128-byte push-constant block, field for field (shaders/sph_common.glsl:10-17,
 * solver/sph.py:116-125). For the splat pass the third row is i_surface
 * (shaders/surface_splat.glsl:14). */
struct glslref_push {
  int32_t i_layout[4];
  int32_t i_grid[4];
  int32_t i_sort[4];
  float f_lo[4];
  float f_hi[4];
  float f_sph[4];
  float f_sim[4];
  int32_t i_collider[4];
};

/* Flat arrays in the reference's texture layout: width 256 texels, RGBA32F for
 * particle/key arrays, R32F for cells and the surface grid
 * (solver/gpu_util.py:28-59, solver/sph.py:127-152). Row counts are
 * ceil(count/256). */
struct glslref_images {
  float *positions, *velocities, *lambda, *predicted, *delta, *normal, *keys;
  float *cell_start, *cell_end, *surface, *collider;
  int32_t particle_rows, key_rows, cell_rows, surface_rows;
  int32_t collider_dims[3];
  int32_t width;
};
}

#define FLOWX_PASS_PRELUDE                                                            \
  ivec4 i_layout, i_grid, i_sort, i_surface, i_collider;                             \
  vec4 f_lo, f_hi, f_sph, f_sim;                                                      \
  image2D positions_img, velocities_img, lambda_img, predicted_img, delta_img,        \
      normal_img, keys_img, cell_start_img, cell_end_img, surface_img;                \
  image3D collider_img;                                                               \
  static thread_local uvec3 gl_GlobalInvocationID;

#define FLOWX_PASS_BIND                                                               \
  static ivec4 to_ivec4(const int32_t *v)                                             \
  {                                                                                   \
    ivec4 r;                                                                          \
    r.x = v[0];                                                                       \
    r.y = v[1];                                                                       \
    r.z = v[2];                                                                       \
    r.w = v[3];                                                                       \
    return r;                                                                         \
  }                                                                                   \
  static vec4 to_vec4(const float *v) { return vec4(v[0], v[1], v[2], v[3]); }        \
  void bind(const glslref_push *pc, const glslref_images *im)                         \
  {                                                                                   \
    i_layout = to_ivec4(pc->i_layout);                                                \
    i_grid = to_ivec4(pc->i_grid);                                                    \
    i_sort = to_ivec4(pc->i_sort);                                                    \
    i_surface = to_ivec4(pc->i_sort);                                                 \
    i_collider = to_ivec4(pc->i_collider);                                            \
    f_lo = to_vec4(pc->f_lo);                                                         \
    f_hi = to_vec4(pc->f_hi);                                                         \
    f_sph = to_vec4(pc->f_sph);                                                       \
    f_sim = to_vec4(pc->f_sim);                                                       \
    const int w = im->width;                                                          \
    positions_img = image2D{im->positions, w, im->particle_rows, 4};                  \
    velocities_img = image2D{im->velocities, w, im->particle_rows, 4};                \
    lambda_img = image2D{im->lambda, w, im->particle_rows, 4};                        \
    predicted_img = image2D{im->predicted, w, im->particle_rows, 4};                  \
    delta_img = image2D{im->delta, w, im->particle_rows, 4};                          \
    normal_img = image2D{im->normal, w, im->particle_rows, 4};                        \
    keys_img = image2D{im->keys, w, im->key_rows, 4};                                 \
    cell_start_img = image2D{im->cell_start, w, im->cell_rows, 1};                    \
    cell_end_img = image2D{im->cell_end, w, im->cell_rows, 1};                        \
    surface_img = image2D{im->surface, w, im->surface_rows, 1};                       \
    collider_img = image3D{im->collider, im->collider_dims[0], im->collider_dims[1],  \
                           im->collider_dims[2]};                                     \
  }                                                                                   \
  void run(int count)                                                                 \
  {                                                                                   \
    _Pragma("omp parallel for schedule(static)") for (int g = 0; g < count; ++g)      \
    {                                                                                 \
      gl_GlobalInvocationID = uvec3{(unsigned)g, 0u, 0u};                             \
      pass_main();                                                                    \
    }                                                                                 \
  }

#define main pass_main

/* One namespace per compiled pass. FLOWX_GLSL_PASS(ns, file) cannot be a macro
 * that takes an #include, so each block is spelled out. */
namespace p_normal {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_normal.glsl"
FLOWX_PASS_BIND
}  // namespace p_normal
namespace p_predict {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_predict.glsl"
FLOWX_PASS_BIND
}  // namespace p_predict
namespace p_grid_key {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_grid_key.glsl"
FLOWX_PASS_BIND
}  // namespace p_grid_key
namespace p_sort {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_sort.glsl"
FLOWX_PASS_BIND
}  // namespace p_sort
namespace p_cell_clear {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_cell_clear.glsl"
FLOWX_PASS_BIND
}  // namespace p_cell_clear
namespace p_cell_range {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_cell_range.glsl"
FLOWX_PASS_BIND
}  // namespace p_cell_range
namespace p_lambda {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_lambda.glsl"
FLOWX_PASS_BIND
}  // namespace p_lambda
namespace p_delta {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_delta.glsl"
FLOWX_PASS_BIND
}  // namespace p_delta
namespace p_apply_delta {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_apply_delta.glsl"
FLOWX_PASS_BIND
}  // namespace p_apply_delta
namespace p_velocity {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_velocity.glsl"
FLOWX_PASS_BIND
}  // namespace p_velocity
namespace p_xsph {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_xsph.glsl"
FLOWX_PASS_BIND
}  // namespace p_xsph
namespace p_finalize {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "sph_finalize.glsl"
FLOWX_PASS_BIND
}  // namespace p_finalize
namespace p_splat {
#include "glsl_shim.h"
FLOWX_PASS_PRELUDE
#include "sph_common.glsl"
#include "surface_splat.glsl"
FLOWX_PASS_BIND
}  // namespace p_splat

#undef main

extern "C" {
/* Pass ids, in the order of solver/sph.py:_PASSES (154-167) plus the splat. */
enum {
  GLSLREF_NORMAL = 0,
  GLSLREF_PREDICT,
  GLSLREF_GRID_KEY,
  GLSLREF_SORT,
  GLSLREF_CELL_CLEAR,
  GLSLREF_CELL_RANGE,
  GLSLREF_LAMBDA,
  GLSLREF_DELTA,
  GLSLREF_APPLY_DELTA,
  GLSLREF_VELOCITY,
  GLSLREF_XSPH,
  GLSLREF_FINALIZE,
  GLSLREF_SPLAT,
};

/* One gpu.compute.dispatch of `invocations` threads (rounded up to whole
 * work groups of 64, like solver/gpu_util.py:157-159). Returns 0, or -1 for an
 * unknown pass id. */
int glslref_dispatch(int pass_id, const glslref_push *pc, const glslref_images *im,
                     int invocations)
{
  const int groups = invocations <= 0 ? 1 : (invocations + 63) / 64;
  const int count = groups * 64;
  switch (pass_id) {
#define FLOWX_CASE(id, ns) \
  case id:                 \
    ns::bind(pc, im);      \
    ns::run(count);        \
    return 0;
    FLOWX_CASE(GLSLREF_NORMAL, p_normal)
    FLOWX_CASE(GLSLREF_PREDICT, p_predict)
    FLOWX_CASE(GLSLREF_GRID_KEY, p_grid_key)
    FLOWX_CASE(GLSLREF_SORT, p_sort)
    FLOWX_CASE(GLSLREF_CELL_CLEAR, p_cell_clear)
    FLOWX_CASE(GLSLREF_CELL_RANGE, p_cell_range)
    FLOWX_CASE(GLSLREF_LAMBDA, p_lambda)
    FLOWX_CASE(GLSLREF_DELTA, p_delta)
    FLOWX_CASE(GLSLREF_APPLY_DELTA, p_apply_delta)
    FLOWX_CASE(GLSLREF_VELOCITY, p_velocity)
    FLOWX_CASE(GLSLREF_XSPH, p_xsph)
    FLOWX_CASE(GLSLREF_FINALIZE, p_finalize)
    FLOWX_CASE(GLSLREF_SPLAT, p_splat)
#undef FLOWX_CASE
    default:
      return -1;
  }
}
}
