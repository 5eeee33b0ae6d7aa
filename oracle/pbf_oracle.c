/* Oracle (test infrastructure only) - never linked into, or called by, the
 * product path. Plain-C float32 restatement of Flow-X's PBF compute passes.
 *
 * Each function restates one GLSL pass of the reference (file:line cited at
 * the function) over flat arrays in the reference's layouts: particle arrays
 * are N x float4, keys S x float4 (key, id, 0, 0) with S = next power of two
 * >= N, cell_start / cell_end C floats with -1 for an empty cell, collider a
 * uint8 occupancy grid x-fastest, splat grid one float per sample.
 *
 * Arithmetic is float32 in the order the GLSL writes it (compiled with
 * -ffp-contract=off), so the only differences from the reference's own source
 * run as C++ (oracle/glsl_cpu) are in how constant expressions round. The grid
 * build offers both the reference's bitonic network (sph_sort.glsl, unstable,
 * ordering by key only) and the stable (key, id) order the CUDA path emits.
 *
 * Parity pinned by tests/test_oracle.py against the golden fixtures of
 * tests/golden/ (generated from the reference's own passes).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.14159265358979323846f
#define MAX_CELL_SCAN 512          /* shaders/sph_common.glsl:30 */
#define MAX_COLLIDER_SEARCH 2      /* shaders/sph_finalize.glsl:13 */
#define SURFACE_CELL_RADIUS 2      /* shaders/surface_splat.glsl:30 */

typedef struct {
  int32_t i_layout[4]; /* N, 256, 256, S */
  int32_t i_grid[4];   /* cells xyz, C */
  int32_t i_sort[4];   /* k, j, bits(scorr), bits(sigma) | splat: samples xyz, bits(spacing) */
  float f_lo[4];       /* lo xyz, cell size */
  float f_hi[4];       /* hi xyz, particle radius | splat: surface lo xyz */
  float f_sph[4];      /* h, mass, rest density, epsilon | splat: kernel radius in x */
  float f_sim[4];      /* viscosity, dt, gravity, damping */
  int32_t i_collider[4];
} oracle_push;

typedef struct {
  float *positions, *velocities, *lambda, *predicted, *delta, *normal, *keys;
  float *cell_start, *cell_end, *surface;
  const uint8_t *collider;
} oracle_buffers;

static float bits_to_float(int32_t b)
{
  float f;
  memcpy(&f, &b, 4);
  return f;
}

/* ---- shaders/sph_common.glsl helpers ----------------------------------- */
typedef struct {
  int x, y, z;
} i3;

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* sph_common.glsl:50-54 */
static i3 cell_coord(const oracle_push *pc, float px, float py, float pz)
{
  i3 g;
  g.x = clampi((int)floorf((px - pc->f_lo[0]) / pc->f_lo[3]), 0, pc->i_grid[0] - 1);
  g.y = clampi((int)floorf((py - pc->f_lo[1]) / pc->f_lo[3]), 0, pc->i_grid[1] - 1);
  g.z = clampi((int)floorf((pz - pc->f_lo[2]) / pc->f_lo[3]), 0, pc->i_grid[2] - 1);
  return g;
}
/* sph_common.glsl:56-59 */
static int cell_index(const oracle_push *pc, i3 g)
{
  return (g.z * pc->i_grid[1] + g.y) * pc->i_grid[0] + g.x;
}
/* sph_common.glsl:61-64 */
static int cell_in_bounds(const oracle_push *pc, i3 g)
{
  return g.x >= 0 && g.y >= 0 && g.z >= 0 && g.x < pc->i_grid[0] && g.y < pc->i_grid[1] &&
         g.z < pc->i_grid[2];
}
/* sph_common.glsl:68-81 */
static float poly6_coef(float h) { return 315.0f / (64.0f * PI_F * powf(h, 9.0f)); }
static float spiky_grad_coef(float h) { return -45.0f / (PI_F * powf(h, 6.0f)); }
static float visc_lap_coef(float h) { return 45.0f / (PI_F * powf(h, 6.0f)); }
/* sph_common.glsl:84-91 */
static float w_poly6(float r2, float h2, float coef)
{
  if (r2 >= h2) return 0.0f;
  float d = h2 - r2;
  return coef * d * d * d;
}
/* sph_common.glsl:111-118 */
static float w_spiky_grad(float r, float h, float coef)
{
  if (r >= h) return 0.0f;
  float d = h - r;
  return coef * d * d;
}
/* sph_common.glsl:121-127 */
static float w_visc_lap(float r, float h, float coef)
{
  if (r >= h) return 0.0f;
  return coef * (h - r);
}
/* sph_common.glsl:139-160 */
static float collider_voxel(const oracle_push *pc) { return bits_to_float(pc->i_collider[3]); }
static i3 collider_coord(const oracle_push *pc, float px, float py, float pz)
{
  float v = collider_voxel(pc);
  i3 c = {(int)floorf((px - pc->f_lo[0]) / v), (int)floorf((py - pc->f_lo[1]) / v),
          (int)floorf((pz - pc->f_lo[2]) / v)};
  return c;
}
static int collider_in_bounds(const oracle_push *pc, i3 c)
{
  return c.x >= 0 && c.y >= 0 && c.z >= 0 && c.x < pc->i_collider[0] && c.y < pc->i_collider[1] &&
         c.z < pc->i_collider[2];
}
static int collider_occupied(const oracle_push *pc, const oracle_buffers *b, i3 c)
{
  if (!collider_in_bounds(pc, c) || !b->collider) return 0;
  return b->collider[((long)c.z * pc->i_collider[1] + c.y) * pc->i_collider[0] + c.x] != 0;
}

/* Iterate the neighbour slots of the (2R+1)^3 cells around `base` in the
 * reference's order (dz, dy, dx, then key slot), MAX_CELL_SCAN per cell. */
#define FOR_NEIGHBOUR_SLOTS(pc, b, base, R, k)                                          \
  for (int dz_ = -(R); dz_ <= (R); ++dz_)                                               \
    for (int dy_ = -(R); dy_ <= (R); ++dy_)                                             \
      for (int dx_ = -(R); dx_ <= (R); ++dx_)                                           \
        for (int cell_ok_ = 1; cell_ok_; cell_ok_ = 0)                                  \
          for (i3 g_ = {(base).x + dx_, (base).y + dy_, (base).z + dz_}; cell_ok_;       \
               cell_ok_ = 0)                                                            \
            if (cell_in_bounds(pc, g_))                                                 \
              for (int c_ = cell_index(pc, g_), start_ = (int)(b)->cell_start[c_],      \
                       end_ = start_ < 0 ? 0                                            \
                                        : ((int)(b)->cell_end[c_] < start_ + MAX_CELL_SCAN \
                                               ? (int)(b)->cell_end[c_]                 \
                                               : start_ + MAX_CELL_SCAN),               \
                       k = start_ < 0 ? 0 : start_;                                     \
                   k < end_; ++k)

/* ---- passes ------------------------------------------------------------- */

/* shaders/sph_normal.glsl:24-81 */
static void pass_normal(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
  const float h = pc->f_sph[0], h2 = h * h, mass = pc->f_sph[1];
  const float poly6 = poly6_coef(h), vlap = visc_lap_coef(h);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    const float *pi = b->predicted + 4 * i;
    float nx = 0, ny = 0, nz = 0, lap = 0;
    i3 base = cell_coord(pc, pi[0], pi[1], pi[2]);
    FOR_NEIGHBOUR_SLOTS(pc, b, base, 1, k)
    {
      int j = (int)b->keys[4 * k + 1];
      if (j == i) continue;
      const float *pj = b->predicted + 4 * j;
      float dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
      float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 >= h2) continue;
      float rho_j = fmaxf(b->lambda[4 * j], 1e-6f);
      float weight = mass / rho_j;
      /* w_poly6_grad, sph_common.glsl:100-107 */
      float t = h2 - r2;
      float s = poly6 * -6.0f * t * t;
      nx += weight * (s * dx);
      ny += weight * (s * dy);
      nz += weight * (s * dz);
      lap += weight * w_visc_lap(sqrtf(r2), h, vlap);
    }
    float mag = sqrtf(nx * nx + ny * ny + nz * nz);
    float curv = (mag > 1e-4f) ? -lap / mag : 0.0f;
    float *o = b->normal + 4 * i;
    o[0] = nx;
    o[1] = ny;
    o[2] = nz;
    o[3] = curv;
  }
}

/* shaders/sph_predict.glsl:23-57 */
static void pass_predict(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
  const float dt = pc->f_sim[1], h = pc->f_sph[0], mass = pc->f_sph[1];
  const float sigma = bits_to_float(pc->i_sort[3]);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    float *v = b->velocities + 4 * i;
    float vx = v[0], vy = v[1], vz = v[2];
    vz += pc->f_sim[2] * dt;
    if (sigma > 0.0f) {
      const float *nn = b->normal + 4 * i;
      float mag = sqrtf(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
      if (mag > 1e-4f) {
        float s = -sigma * nn[3];
        vx += ((s * nn[0]) / mag / mass) * dt;
        vy += ((s * nn[1]) / mag / mass) * dt;
        vz += ((s * nn[2]) / mag / mass) * dt;
      }
    }
    float v_max = 0.4f * h / fmaxf(dt, 1e-6f);
    float speed = sqrtf(vx * vx + vy * vy + vz * vz);
    if (speed > v_max) {
      float s = v_max / speed;
      vx *= s;
      vy *= s;
      vz *= s;
    }
    const float *p = b->positions + 4 * i;
    float *q = b->predicted + 4 * i;
    q[0] = p[0] + vx * dt;
    q[1] = p[1] + vy * dt;
    q[2] = p[2] + vz * dt;
    q[3] = 1.0f;
    v[0] = vx;
    v[1] = vy;
    v[2] = vz;
    v[3] = 0.0f;
  }
}

/* shaders/sph_grid_key.glsl:14-28 */
static void pass_grid_key(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0], s = pc->i_layout[3];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s; ++i) {
    float key = (float)pc->i_grid[3];
    if (i < n) {
      const float *p = b->predicted + 4 * i;
      key = (float)cell_index(pc, cell_coord(pc, p[0], p[1], p[2]));
    }
    float *k = b->keys + 4 * i;
    k[0] = key;
    k[1] = (float)i;
    k[2] = 0.0f;
    k[3] = 0.0f;
  }
}

/* shaders/sph_sort.glsl:14-34, one (k, j) compare-exchange step. */
static void pass_sort_step(const oracle_push *pc, oracle_buffers *b)
{
  const int s = pc->i_layout[3], kk = pc->i_sort[0], jj = pc->i_sort[1];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s; ++i) {
    int partner = i ^ jj;
    if (partner <= i) continue;
    float *a = b->keys + 4 * i, *c = b->keys + 4 * partner;
    int ascending = (i & kk) == 0;
    if ((a[0] > c[0]) == ascending) {
      float tmp[4];
      memcpy(tmp, a, 16);
      memcpy(a, c, 16);
      memcpy(c, tmp, 16);
    }
  }
}

/* shaders/sph_cell_clear.glsl:8-16 */
static void pass_cell_clear(const oracle_push *pc, oracle_buffers *b)
{
  const int c = pc->i_grid[3];
  for (int i = 0; i < c; ++i) {
    b->cell_start[i] = -1.0f;
    b->cell_end[i] = -1.0f;
  }
}

/* shaders/sph_cell_range.glsl:10-32 */
static void pass_cell_range(const oracle_push *pc, oracle_buffers *b)
{
  const int s = pc->i_layout[3];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s; ++i) {
    int key = (int)b->keys[4 * i];
    if (key >= pc->i_grid[3]) continue;
    int prev = (i == 0) ? -1 : (int)b->keys[4 * (i - 1)];
    int next = (i == s - 1) ? -1 : (int)b->keys[4 * (i + 1)];
    if (key != prev) b->cell_start[key] = (float)i;
    if (key != next) b->cell_end[key] = (float)(i + 1);
  }
}

/* shaders/sph_lambda.glsl:17-77 */
static void pass_lambda(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
  const float h = pc->f_sph[0], h2 = h * h, mass = pc->f_sph[1], rest = pc->f_sph[2];
  const float eps = pc->f_sph[3], poly6 = poly6_coef(h), spiky = spiky_grad_coef(h);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    const float *pi = b->predicted + 4 * i;
    float density = 0, gx = 0, gy = 0, gz = 0, gn2 = 0;
    i3 base = cell_coord(pc, pi[0], pi[1], pi[2]);
    FOR_NEIGHBOUR_SLOTS(pc, b, base, 1, k)
    {
      int j = (int)b->keys[4 * k + 1];
      const float *pj = b->predicted + 4 * j;
      float dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
      float r2 = dx * dx + dy * dy + dz * dz;
      density += mass * w_poly6(r2, h2, poly6);
      if (j == i || r2 >= h2 || r2 <= 1e-12f) continue;
      float r = sqrtf(r2);
      float s = mass * w_spiky_grad(r, h, spiky);
      float ax = s * (dx / r), ay = s * (dy / r), az = s * (dz / r);
      gx += ax;
      gy += ay;
      gz += az;
      gn2 += ax * ax + ay * ay + az * az;
    }
    float constraint = fmaxf(density, 1e-6f) / rest - 1.0f;
    float denom = (gx * gx + gy * gy + gz * gz + gn2) / (rest * rest) + eps;
    float lam = -constraint / fmaxf(denom, 1e-9f);
    float *o = b->lambda + 4 * i;
    o[0] = fmaxf(density, 1e-6f);
    o[1] = lam;
    o[2] = 0.0f;
    o[3] = 0.0f;
  }
}

/* shaders/sph_delta.glsl:19-85 */
static void pass_delta(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
  const float h = pc->f_sph[0], h2 = h * h, rest = pc->f_sph[2];
  const float spiky = spiky_grad_coef(h), poly6 = poly6_coef(h);
  const float scorr_k = bits_to_float(pc->i_sort[2]);
  const float q = 0.2f * h;
  const float w_q = w_poly6(q * q, h2, poly6);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    const float *pi = b->predicted + 4 * i;
    const float lambda_i = b->lambda[4 * i + 1];
    float ax = 0, ay = 0, az = 0;
    i3 base = cell_coord(pc, pi[0], pi[1], pi[2]);
    FOR_NEIGHBOUR_SLOTS(pc, b, base, 1, k)
    {
      int j = (int)b->keys[4 * k + 1];
      if (j == i) continue;
      const float *pj = b->predicted + 4 * j;
      float dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
      float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 >= h2 || r2 <= 1e-12f) continue;
      float r = sqrtf(r2);
      float lambda_j = b->lambda[4 * j + 1];
      float s_corr = 0.0f;
      if (scorr_k > 0.0f && w_q > 1e-9f) {
        float ratio = w_poly6(r2, h2, poly6) / w_q;
        float rr = fmaxf(ratio, 0.0f);
        /* pow(max(ratio, 0), 4.0) (sph_delta.glsl:75), evaluated as two
         * squarings: GLSL leaves pow's accuracy to the implementation and
         * an integer power is exact to within one rounding this way. */
        float rr2 = rr * rr;
        s_corr = -scorr_k * (rr2 * rr2);
      }
      float s = (lambda_i + lambda_j + s_corr) * w_spiky_grad(r, h, spiky);
      ax += s * (dx / r);
      ay += s * (dy / r);
      az += s * (dz / r);
    }
    float *o = b->delta + 4 * i;
    o[0] = ax / rest;
    o[1] = ay / rest;
    o[2] = az / rest;
    o[3] = 0.0f;
  }
}

/* shaders/sph_apply_delta.glsl:10-20 */
static void pass_apply_delta(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    float *p = b->predicted + 4 * i;
    const float *d = b->delta + 4 * i;
    p[0] = p[0] + d[0];
    p[1] = p[1] + d[1];
    p[2] = p[2] + d[2];
    p[3] = 1.0f;
  }
}

/* shaders/sph_velocity.glsl:12-24 */
static void pass_velocity(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
  const float dtc = fmaxf(pc->f_sim[1], 1e-6f);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const float *q = b->predicted + 4 * i, *p = b->positions + 4 * i;
    float *v = b->velocities + 4 * i;
    v[0] = (q[0] - p[0]) / dtc;
    v[1] = (q[1] - p[1]) / dtc;
    v[2] = (q[2] - p[2]) / dtc;
    v[3] = 0.0f;
  }
}

/* shaders/sph_xsph.glsl:28-82 */
static void pass_xsph(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
  const float h = pc->f_sph[0], h2 = h * h, mass = pc->f_sph[1], poly6 = poly6_coef(h);
  const float c = pc->f_sim[0];
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    const float *pi = b->predicted + 4 * i, *vi = b->velocities + 4 * i;
    float ax = 0, ay = 0, az = 0;
    i3 base = cell_coord(pc, pi[0], pi[1], pi[2]);
    FOR_NEIGHBOUR_SLOTS(pc, b, base, 1, k)
    {
      int j = (int)b->keys[4 * k + 1];
      if (j == i) continue;
      const float *pj = b->predicted + 4 * j;
      float dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
      float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 >= h2) continue;
      float rho_j = fmaxf(b->lambda[4 * j], 1e-6f);
      const float *vj = b->velocities + 4 * j;
      float w = (mass / rho_j);
      float wk = w_poly6(r2, h2, poly6);
      ax += (w * (vj[0] - vi[0])) * wk;
      ay += (w * (vj[1] - vi[1])) * wk;
      az += (w * (vj[2] - vi[2])) * wk;
    }
    float *o = b->delta + 4 * i;
    o[0] = c * ax;
    o[1] = c * ay;
    o[2] = c * az;
    o[3] = 0.0f;
  }
}

/* shaders/sph_finalize.glsl:13-96 */
static void pass_finalize(const oracle_push *pc, oracle_buffers *b)
{
  const int n = pc->i_layout[0];
  const float radius = pc->f_hi[3], damping = pc->f_sim[3];
  const float voxel = collider_voxel(pc);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    float *vv = b->velocities + 4 * i;
    const float *dd = b->delta + 4 * i;
    const float *q = b->predicted + 4 * i;
    float v[3] = {vv[0] + dd[0], vv[1] + dd[1], vv[2] + dd[2]};
    float p[3] = {q[0], q[1], q[2]};
    if (voxel > 0.0f && collider_occupied(pc, b, collider_coord(pc, p[0], p[1], p[2]))) {
      float best[3] = {0, 0, 0}, best_d2 = 1e30f;
      int found = 0;
      i3 c = collider_coord(pc, p[0], p[1], p[2]);
      for (int dz = -MAX_COLLIDER_SEARCH; dz <= MAX_COLLIDER_SEARCH; ++dz)
        for (int dy = -MAX_COLLIDER_SEARCH; dy <= MAX_COLLIDER_SEARCH; ++dy)
          for (int dx = -MAX_COLLIDER_SEARCH; dx <= MAX_COLLIDER_SEARCH; ++dx) {
            i3 nc = {c.x + dx, c.y + dy, c.z + dz};
            if (!collider_in_bounds(pc, nc) || collider_occupied(pc, b, nc)) continue;
            float cx = pc->f_lo[0] + ((float)nc.x + 0.5f) * voxel;
            float cy = pc->f_lo[1] + ((float)nc.y + 0.5f) * voxel;
            float cz = pc->f_lo[2] + ((float)nc.z + 0.5f) * voxel;
            float ex = cx - p[0], ey = cy - p[1], ez = cz - p[2];
            float d2 = ex * ex + ey * ey + ez * ez;
            if (d2 < best_d2) {
              best_d2 = d2;
              best[0] = cx;
              best[1] = cy;
              best[2] = cz;
              found = 1;
            }
          }
      if (found) {
        float dist = sqrtf(best_d2);
        float u[3];
        if (dist > 1e-6f) {
          u[0] = (best[0] - p[0]) / dist;
          u[1] = (best[1] - p[1]) / dist;
          u[2] = (best[2] - p[2]) / dist;
        } else {
          u[0] = 0.0f;
          u[1] = 0.0f;
          u[2] = 1.0f;
        }
        float push = dist + radius;
        p[0] += u[0] * push;
        p[1] += u[1] * push;
        p[2] += u[2] * push;
        float vn = v[0] * u[0] + v[1] * u[1] + v[2] * u[2];
        if (vn < 0.0f) {
          float s = vn * (1.0f + damping);
          v[0] -= s * u[0];
          v[1] -= s * u[1];
          v[2] -= s * u[2];
        }
      }
    }
    for (int a = 0; a < 3; ++a) {
      float lo = pc->f_lo[a] + radius, hi = pc->f_hi[a] - radius;
      if (p[a] < lo) {
        p[a] = lo;
        v[a] = -v[a] * damping;
      } else if (p[a] > hi) {
        p[a] = hi;
        v[a] = -v[a] * damping;
      }
    }
    float *po = b->positions + 4 * i;
    po[0] = p[0];
    po[1] = p[1];
    po[2] = p[2];
    po[3] = 1.0f;
    vv[0] = v[0];
    vv[1] = v[1];
    vv[2] = v[2];
    vv[3] = 0.0f;
  }
}

/* shaders/surface_splat.glsl:32-97 (push slots repurposed, :14-24) */
static void pass_splat(const oracle_push *pc, oracle_buffers *b)
{
  const int sx = pc->i_sort[0], sy = pc->i_sort[1], sz = pc->i_sort[2];
  const long samples = (long)sx * sy * sz;
  const float spacing = bits_to_float(pc->i_sort[3]);
  const float h = pc->f_sph[0], h2 = h * h, mass = pc->f_sph[1], rest = pc->f_sph[2];
  const float coef = poly6_coef(h);
  const float voxel = collider_voxel(pc);
#pragma omp parallel for schedule(dynamic, 1024)
  for (long s = 0; s < samples; ++s) {
    int gx = (int)(s % sx), gy = (int)((s / sx) % sy), gz = (int)(s / ((long)sx * sy));
    float px = pc->f_hi[0] + (float)gx * spacing;
    float py = pc->f_hi[1] + (float)gy * spacing;
    float pz = pc->f_hi[2] + (float)gz * spacing;
    float density = 0.0f;
    i3 base = cell_coord(pc, px, py, pz);
    FOR_NEIGHBOUR_SLOTS(pc, b, base, SURFACE_CELL_RADIUS, k)
    {
      int j = (int)b->keys[4 * k + 1];
      const float *pj = b->positions + 4 * j;
      float dx = px - pj[0], dy = py - pj[1], dz = pz - pj[2];
      density += mass * w_poly6(dx * dx + dy * dy + dz * dz, h2, coef);
    }
    float value = density / fmaxf(rest, 1e-6f);
    if (voxel > 0.0f && collider_occupied(pc, b, collider_coord(pc, px, py, pz))) value = 0.0f;
    b->surface[s] = value;
  }
}

/* ---- grid build and the whole substep ------------------------------------ */

typedef struct {
  float key, id;
} key_pair;

static int cmp_key_id(const void *a, const void *b)
{
  const float *x = (const float *)a, *y = (const float *)b;
  if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
  if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
  return 0;
}

enum { ORACLE_ORDER_BITONIC = 0, ORACLE_ORDER_STABLE = 1 };

/* solver/sph.py:482-498 (_build_grid). order selects the reference's bitonic
 * network or the stable (key, id) order. */
void oracle_build_grid(const oracle_push *pc_in, oracle_buffers *b, int order)
{
  oracle_push pc = *pc_in;
  const int s = pc.i_layout[3];
  pass_grid_key(&pc, b);
  if (order == ORACLE_ORDER_BITONIC) {
    for (int k = 2; k <= s; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        pc.i_sort[0] = k;
        pc.i_sort[1] = j;
        pass_sort_step(&pc, b);
      }
    pc.i_sort[0] = pc_in->i_sort[0];
    pc.i_sort[1] = pc_in->i_sort[1];
  } else {
    qsort(b->keys, (size_t)s, 16, cmp_key_id);
  }
  pass_cell_clear(&pc, b);
  pass_cell_range(&pc, b);
}

enum {
  ORACLE_NORMAL = 0,
  ORACLE_PREDICT,
  ORACLE_GRID_KEY,
  ORACLE_SORT,
  ORACLE_CELL_CLEAR,
  ORACLE_CELL_RANGE,
  ORACLE_LAMBDA,
  ORACLE_DELTA,
  ORACLE_APPLY_DELTA,
  ORACLE_VELOCITY,
  ORACLE_XSPH,
  ORACLE_FINALIZE,
  ORACLE_SPLAT,
};

/* One pass by id (same numbering as the CUDA path's pass ids). */
int oracle_pass(int pass_id, const oracle_push *pc, oracle_buffers *b)
{
  switch (pass_id) {
    case ORACLE_NORMAL: pass_normal(pc, b); return 0;
    case ORACLE_PREDICT: pass_predict(pc, b); return 0;
    case ORACLE_GRID_KEY: pass_grid_key(pc, b); return 0;
    case ORACLE_SORT: pass_sort_step(pc, b); return 0;
    case ORACLE_CELL_CLEAR: pass_cell_clear(pc, b); return 0;
    case ORACLE_CELL_RANGE: pass_cell_range(pc, b); return 0;
    case ORACLE_LAMBDA: pass_lambda(pc, b); return 0;
    case ORACLE_DELTA: pass_delta(pc, b); return 0;
    case ORACLE_APPLY_DELTA: pass_apply_delta(pc, b); return 0;
    case ORACLE_VELOCITY: pass_velocity(pc, b); return 0;
    case ORACLE_XSPH: pass_xsph(pc, b); return 0;
    case ORACLE_FINALIZE: pass_finalize(pc, b); return 0;
    case ORACLE_SPLAT: pass_splat(pc, b); return 0;
    default: return -1;
  }
}

/* solver/sph.py:501-514 (_substep), with `iterations` Jacobi iterations. */
void oracle_substep(const oracle_push *pc, oracle_buffers *b, int iterations, int order)
{
  if (bits_to_float(pc->i_sort[3]) > 0.0f) pass_normal(pc, b);
  pass_predict(pc, b);
  oracle_build_grid(pc, b, order);
  for (int it = 0; it < iterations; ++it) {
    pass_lambda(pc, b);
    pass_delta(pc, b);
    pass_apply_delta(pc, b);
  }
  pass_velocity(pc, b);
  pass_xsph(pc, b);
  pass_finalize(pc, b);
}

/* Thread count used by the OpenMP loops (0 = library default). */
#ifdef _OPENMP
#include <omp.h>
void oracle_set_threads(int n)
{
  if (n > 0) omp_set_num_threads(n);
}
int oracle_max_threads(void) { return omp_get_max_threads(); }
#else
void oracle_set_threads(int n) { (void)n; }
int oracle_max_threads(void) { return 1; }
#endif
