// Per-particle and per-pair arithmetic of the PBF passes, shared by the fused
// substep kernels and the single-pass kernels so both evaluate exactly the
// same float32 expressions. Each helper follows the reference pass it cites,
// operation for operation (the library is compiled without FMA contraction,
// so these are the reference's roundings, not a re-association of them).
#pragma once

#include "flowx_internal.cuh"

namespace flowx {

// shaders/sph_predict.glsl:30-56: external force, cohesion, speed clamp, predict.
__device__ __forceinline__ void predict_particle(const SegParams &s, float4 p, float4 v, float4 n,
                                                 float3 &vo, float3 &q)
{
  const float dt = s.dt;
  float vx = v.x, vy = v.y, vz = v.z;
  vz += s.gravity * dt;
  if (s.sigma > 0.0f) {
    float mag = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    if (mag > 1e-4f) {
      float sc = -s.sigma * n.w;
      vx += ((sc * n.x) / mag / s.mass) * dt;
      vy += ((sc * n.y) / mag / s.mass) * dt;
      vz += ((sc * n.z) / mag / s.mass) * dt;
    }
  }
  float speed = sqrtf(vx * vx + vy * vy + vz * vz);
  if (speed > s.v_max) {
    float f = s.v_max / speed;
    vx *= f;
    vy *= f;
    vz *= f;
  }
  vo = make_float3(vx, vy, vz);
  q = make_float3(p.x + vx * dt, p.y + vy * dt, p.z + vz * dt);
}

// shaders/sph_finalize.glsl:22-95 for one particle: collider push-out to the
// nearest free voxel centre within MAX_COLLIDER_SEARCH, then the box clamp.
__device__ __forceinline__ void finalize_particle(const SegParams &s, const uint8_t *__restrict__ col, float3 &p,
                                                  float3 &v)
{
  const float voxel = s.voxel;
  if (voxel > 0.0f) {
    int3 c = collider_coord(s, p.x, p.y, p.z);
    if (collider_occupied(s, col, c.x, c.y, c.z)) {
      float bx = 0.0f, by = 0.0f, bz = 0.0f, best = 1e30f;
      bool found = false;
      for (int dz = -kMaxColliderSearch; dz <= kMaxColliderSearch; ++dz)
        for (int dy = -kMaxColliderSearch; dy <= kMaxColliderSearch; ++dy)
          for (int dx = -kMaxColliderSearch; dx <= kMaxColliderSearch; ++dx) {
            int nx = c.x + dx, ny = c.y + dy, nz = c.z + dz;
            if (nx < 0 || ny < 0 || nz < 0 || nx >= s.col_nx || ny >= s.col_ny || nz >= s.col_nz) continue;
            if (collider_occupied(s, col, nx, ny, nz)) continue;
            float cx = s.lox + ((float)nx + 0.5f) * voxel;
            float cy = s.loy + ((float)ny + 0.5f) * voxel;
            float cz = s.loz + ((float)nz + 0.5f) * voxel;
            float ex = cx - p.x, ey = cy - p.y, ez = cz - p.z;
            float d2 = ex * ex + ey * ey + ez * ez;
            if (d2 < best) {
              best = d2;
              bx = cx;
              by = cy;
              bz = cz;
              found = true;
            }
          }
      if (found) {
        float dist = sqrtf(best);
        float ux, uy, uz;
        if (dist > 1e-6f) {
          ux = (bx - p.x) / dist;
          uy = (by - p.y) / dist;
          uz = (bz - p.z) / dist;
        } else {
          ux = 0.0f;
          uy = 0.0f;
          uz = 1.0f;
        }
        float push = dist + s.radius;
        p.x += ux * push;
        p.y += uy * push;
        p.z += uz * push;
        float vn = v.x * ux + v.y * uy + v.z * uz;
        if (vn < 0.0f) {
          float f = vn * (1.0f + s.damping);
          v.x -= f * ux;
          v.y -= f * uy;
          v.z -= f * uz;
        }
      }
    }
  }
  const float r = s.radius, damp = s.damping;
  float lo, hi;
  lo = s.lox + r; hi = s.hix - r;
  if (p.x < lo) { p.x = lo; v.x = -v.x * damp; } else if (p.x > hi) { p.x = hi; v.x = -v.x * damp; }
  lo = s.loy + r; hi = s.hiy - r;
  if (p.y < lo) { p.y = lo; v.y = -v.y * damp; } else if (p.y > hi) { p.y = hi; v.y = -v.y * damp; }
  lo = s.loz + r; hi = s.hiz - r;
  if (p.z < lo) { p.z = lo; v.z = -v.z * damp; } else if (p.z > hi) { p.z = hi; v.z = -v.z * damp; }
}

// shaders/sph_lambda.glsl:53-74 for particle i at slot i.
__device__ __forceinline__ float2 lambda_particle(const SegParams &s, const uint32_t *__restrict__ off,
                                                  const float4 *__restrict__ pred, int i)
{
  const float4 pi = pred[i];
  const float h = s.h, h2 = s.h2, mass = s.mass, poly6 = s.poly6, spiky = s.spiky;
  float density = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f, gn2 = 0.0f;
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  for_each_candidate<1>(s, off, base, [&](int k) {
    const float4 pj = __ldg(&pred[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    density += mass * w_poly6(r2, h2, poly6);
    if (k == i || r2 >= h2 || r2 <= 1e-12f) return;
    const float r = sqrtf(r2);
    const float sg = mass * w_spiky_grad(r, h, spiky);
    const float ax = sg * (dx / r), ay = sg * (dy / r), az = sg * (dz / r);
    gx += ax;
    gy += ay;
    gz += az;
    gn2 += ax * ax + ay * ay + az * az;
  });
  const float rest = s.rest;
  const float constraint = fmaxf(density, 1e-6f) / rest - 1.0f;
  const float denom = (gx * gx + gy * gy + gz * gz + gn2) / (rest * rest) + s.eps;
  const float lam = -constraint / fmaxf(denom, 1e-9f);
  return make_float2(fmaxf(density, 1e-6f), lam);
}

// shaders/sph_delta.glsl:29-84: the position correction before the 1/rho0
// scale, returned as the summed vector; callers divide by rest density.
__device__ __forceinline__ float3 delta_sum(const SegParams &s, const uint32_t *__restrict__ off,
                                            const float4 *__restrict__ pred, const float2 *__restrict__ lam,
                                            int i)
{
  const float4 pi = pred[i];
  const float lambda_i = lam[i].y;
  const float h = s.h, h2 = s.h2, spiky = s.spiky, poly6 = s.poly6, scorr_k = s.scorr_k, w_q = s.w_q;
  const bool use_scorr = scorr_k > 0.0f && w_q > 1e-9f;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  for_each_candidate<1>(s, off, base, [&](int k) {
    if (k == i) return;
    const float4 pj = __ldg(&pred[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 >= h2 || r2 <= 1e-12f) return;
    const float r = sqrtf(r2);
    const float lambda_j = __ldg(&lam[k].y);
    float s_corr = 0.0f;
    if (use_scorr) {
      const float ratio = w_poly6(r2, h2, poly6) / w_q;
      const float rr = fmaxf(ratio, 0.0f);
      const float rr2 = rr * rr;
      s_corr = -scorr_k * (rr2 * rr2);
    }
    const float sc = (lambda_i + lambda_j + s_corr) * w_spiky_grad(r, h, spiky);
    ax += sc * (dx / r);
    ay += sc * (dy / r);
    az += sc * (dz / r);
  });
  return make_float3(ax, ay, az);
}

// shaders/sph_normal.glsl:31-79 for particle i.
__device__ __forceinline__ float4 normal_particle(const SegParams &s, const uint32_t *__restrict__ off,
                                                  const float4 *__restrict__ pred, const float2 *__restrict__ lam,
                                                  int i)
{
  const float4 pi = pred[i];
  const float h = s.h, h2 = s.h2, mass = s.mass, poly6m6 = s.poly6m6, vlap = s.visclap;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f, lap = 0.0f;
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  for_each_candidate<1>(s, off, base, [&](int k) {
    if (k == i) return;
    const float4 pj = __ldg(&pred[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 >= h2) return;
    const float rho_j = fmaxf(__ldg(&lam[k].x), 1e-6f);
    const float weight = mass / rho_j;
    const float t = h2 - r2;
    const float sg = poly6m6 * t * t;
    nx += weight * (sg * dx);
    ny += weight * (sg * dy);
    nz += weight * (sg * dz);
    lap += weight * w_visc_lap(sqrtf(r2), h, vlap);
  });
  const float mag = sqrtf(nx * nx + ny * ny + nz * nz);
  const float curv = (mag > 1e-4f) ? -lap / mag : 0.0f;
  return make_float4(nx, ny, nz, curv);
}

}  // namespace flowx
