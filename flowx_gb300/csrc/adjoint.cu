// Differentiable substeps: a checkpointed forward of the fused substep in
// particle-id order and its hand-written adjoint (C ABI in include/flowx.h).
// No reference counterpart: Flow-X's solver is not differentiable.
//
// Forward (solver/sph.py:501-514, the float32 expressions of the reference's
// passes as pbf_math.cuh evaluates them): particle arrays stay in id order and
// every neighbour walk visits the grid's sorted id column, cell by cell in
// the reference's (dz, dy, dx, slot) order, so the trajectory is the one the
// fused path computes with FLOWX_FLAG_EXACT. Per substep s the state entering
// it (positions, velocities, predicted, last densities) is checkpointed and
// the grid the substep builds is kept (sorted ids, cell offsets, each
// particle's cell and slot).
//
// Adjoint, substep by substep from the last: the substep is recomputed from
// its checkpoint with every Jacobi iterate kept, then reversed pass by pass:
//   finalize  - box clamp and collider push-out of the branch taken;
//   xsph      - through the velocities, the neighbour densities and W;
//   velocity  - v = (p - x) / dt;
//   I x { delta  - through lambda_i, lambda_j, s_corr and the spiky gradient;
//         lambda - through C_i, the denominator (|sum g|^2 + sum |g|^2) and
//                  the density }, last iteration first;
//   predict   - speed clamp and the cohesion force from (normal, curvature);
//   normal    - the previous substep's grid, predicted positions and densities.
// A neighbour pass's contribution to a partner j is added with a float4
// atomic, so gradients are reproducible to float32 rounding, not bitwise.
// The grid is not differentiated: a particle's candidate set is fixed by the
// cells it was sorted into.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "runtime.h"
#include "pbf_math.cuh"

namespace flowx {
namespace {

constexpr int kBlock = 128;
constexpr int kMaxIterations = 1000;  // as flowx_substep accepts

inline unsigned blocks_for(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

// One substep's neighbour grid in id order: sorted ids per slot, cell
// offsets, and per particle id its cell and its slot.
struct GridView {
  const uint32_t *ids;   // [slot]
  const uint32_t *off;   // [cell], cells + 1
  const uint32_t *cell;  // [id]
  const uint32_t *slot;  // [id]
};

// Splat parameters (surface_splat.glsl:32-97 with the push slots of
// solver/surface.py:201-239).
struct SplatGeom {
  float slox, sloy, sloz, spacing;
  float kr, kh2, kcoef, mass, rest;
  int snx, sny, snz;
};

// Candidates of the (2R+1)^3 cells around `base` as particle ids.
template <int R, class F>
__device__ __forceinline__ void for_each_id(const SegParams &s, const GridView &g, int3 base, F &&f)
{
  for_each_candidate<R>(s, g.off, base, [&](int k) { f((int)__ldg(&g.ids[k])); });
}

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 scale3(float3 a, float k) { return make_float3(a.x * k, a.y * k, a.z * k); }
__device__ __forceinline__ void atomic_add3(float4 *p, float3 v) { atomicAdd(p, make_float4(v.x, v.y, v.z, 0.0f)); }

// J_phi^T y for phi(d) = (h - r)^2 d / r (symmetric Jacobian):
// (h - r)^2 / r * y - (h - r)(h + r) / r^3 * d (d . y).
__device__ __forceinline__ float3 jphi(float3 d, float r, float h, float3 y)
{
  const float hr = h - r;
  const float a = hr * hr / r;
  const float b = hr * (h + r) / (r * r * r);
  return sub3(scale3(y, a), scale3(d, b * dot3(d, y)));
}

// ---- warp-per-particle neighbour walks ---------------------------------------
// At the sizes this path serves (tens of thousands of particles) one thread
// per particle leaves the SMs nearly empty and every candidate costs two
// dependent loads (sorted id, then position). So a warp takes one particle:
// each run of candidate slots goes 32 at a time, one candidate per lane, and
// the lanes' terms are added in slot order (lowest lane first) with
// shuffles. Every term is computed by the same float32 expression as the
// sequential loop and added in the same order, so forward sums equal the
// sequential ones bit for bit; reverse passes reduce their own-particle sums
// with a shuffle tree (order free) and add partner terms with atomics.
constexpr unsigned kFull = 0xffffffffu;

inline unsigned warp_blocks(long long n) { return (unsigned)((n * 32 + kBlock - 1) / kBlock); }

// The candidate runs of the (2R+1)^3 cells around `base` in the reference's
// order: one run per (dz, dy) row, or one per cell (capped at kMaxCellScan)
// when the row holds more than kMaxCellScan slots (as for_each_candidate).
template <int R, class F>
__device__ __forceinline__ void for_each_run(const SegParams &s, const uint32_t *__restrict__ off, int3 base, F &&f)
{
#pragma unroll 1
  for (int dz = -R; dz <= R; ++dz) {
    const int z = base.z + dz;
    if (z < 0 || z >= s.nz) continue;
#pragma unroll 1
    for (int dy = -R; dy <= R; ++dy) {
      const int y = base.y + dy;
      if (y < 0 || y >= s.ny) continue;
      const int x0 = max(base.x - R, 0), x1 = min(base.x + R, s.nx - 1);
      const int row = s.c_begin + (z * s.ny + y) * s.nx;
      const uint32_t a = __ldg(&off[row + x0]);
      const uint32_t b = __ldg(&off[row + x1 + 1]);
      if (b - a <= (uint32_t)kMaxCellScan) {
        f(a, b);
      } else {
#pragma unroll 1
        for (int x = x0; x <= x1; ++x) {
          const uint32_t cs = __ldg(&off[row + x]);
          uint32_t ce = __ldg(&off[row + x + 1]);
          if (ce - cs > (uint32_t)kMaxCellScan) ce = cs + kMaxCellScan;
          f(cs, ce);
        }
      }
    }
  }
}

// f(valid, j) on every lane of the warp for each chunk of 32 candidate slots,
// lane l holding slot chunk + l (j = its particle id, -1 past the run).
template <int R, class F>
__device__ __forceinline__ void warp_chunks(const SegParams &s, const GridView &g, int3 base, int lane, F &&f)
{
  for_each_run<R>(s, g.off, base, [&](uint32_t a, uint32_t b) {
#pragma unroll 1
    for (uint32_t c = a; c < b; c += 32) {
      const uint32_t k = c + (uint32_t)lane;
      const bool valid = k < b;
      f(valid, valid ? (int)__ldg(&g.ids[k]) : -1);
    }
  });
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// ---- forward passes (id order) ---------------------------------------------

// sph_normal.glsl:24-81 over the previous substep's grid.
__global__ void __launch_bounds__(kBlock) k_ad_normal(const SegParams *__restrict__ segs, GridView g,
                                                      const float4 *__restrict__ pred,
                                                      const float *__restrict__ rho, int n,
                                                      float4 *__restrict__ out)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float4 pi = pred[i];
  const float h = s.h, h2 = s.h2, mass = s.mass, poly6m6 = s.poly6m6, vlap = s.visclap;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f, lap = 0.0f;
  warp_chunks<1>(s, g, cell_coord(s, pi.x, pi.y, pi.z), lane, [&](bool valid, int j) {
    float tx = 0.0f, ty = 0.0f, tz = 0.0f, tl = 0.0f;
    bool take = false;
    if (valid && j != i) {
      const float4 pj = __ldg(&pred[j]);
      const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < h2) {
        const float rho_j = fmaxf(__ldg(&rho[j]), 1e-6f);
        const float weight = mass / rho_j;
        const float t = h2 - r2;
        const float sg = poly6m6 * t * t;
        tx = weight * (sg * dx);
        ty = weight * (sg * dy);
        tz = weight * (sg * dz);
        tl = weight * w_visc_lap(sqrtf(r2), h, vlap);
        take = true;
      }
    }
    unsigned m = __ballot_sync(kFull, take);
    while (m) {
      const int t = __ffs(m) - 1;
      m &= m - 1;
      nx += __shfl_sync(kFull, tx, t);
      ny += __shfl_sync(kFull, ty, t);
      nz += __shfl_sync(kFull, tz, t);
      lap += __shfl_sync(kFull, tl, t);
    }
  });
  if (lane == 0) {
    const float mag = sqrtf(nx * nx + ny * ny + nz * nz);
    const float curv = (mag > 1e-4f) ? -lap / mag : 0.0f;
    out[i] = make_float4(nx, ny, nz, curv);
  }
}

// sph_predict.glsl:23-57
__global__ void __launch_bounds__(kBlock) k_ad_predict(const SegParams *__restrict__ segs,
                                                       const float4 *__restrict__ pos,
                                                       const float4 *__restrict__ vel,
                                                       const float4 *__restrict__ normal, int n,
                                                       float4 *__restrict__ q_out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float4 nn = s.sigma > 0.0f ? normal[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  float3 vo, q;
  predict_particle(s, pos[i], vel[i], nn, vo, q);
  q_out[i] = make_float4(q.x, q.y, q.z, 1.0f);
}

// sph_lambda.glsl:17-77; also keeps (sum g, sum |g|^2) for the adjoint.
__global__ void __launch_bounds__(kBlock) k_ad_lambda(const SegParams *__restrict__ segs, GridView g,
                                                      const float4 *__restrict__ pred, int n,
                                                      float2 *__restrict__ lam, float4 *__restrict__ sq)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float4 pi = pred[i];
  const float h = s.h, h2 = s.h2, mass = s.mass, poly6 = s.poly6, spiky = s.spiky;
  float density = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f, gn2 = 0.0f;
  warp_chunks<1>(s, g, cell_coord(s, pi.x, pi.y, pi.z), lane, [&](bool valid, int j) {
    float td = 0.0f, ax = 0.0f, ay = 0.0f, az = 0.0f, an = 0.0f;
    bool dens = false, grad = false;
    if (valid) {
      const float4 pj = __ldg(&pred[j]);
      const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < h2) {  // out of range the sequential loop adds mass * 0
        td = mass * w_poly6(r2, h2, poly6);
        dens = true;
      }
      if (j != i && r2 < h2 && r2 > 1e-12f) {
        const float r = sqrtf(r2);
        const float sg = mass * w_spiky_grad(r, h, spiky);
        ax = sg * (dx / r);
        ay = sg * (dy / r);
        az = sg * (dz / r);
        an = ax * ax + ay * ay + az * az;
        grad = true;
      }
    }
    unsigned m = __ballot_sync(kFull, dens);
    while (m) {
      const int t = __ffs(m) - 1;
      m &= m - 1;
      density += __shfl_sync(kFull, td, t);
    }
    m = __ballot_sync(kFull, grad);
    while (m) {
      const int t = __ffs(m) - 1;
      m &= m - 1;
      gx += __shfl_sync(kFull, ax, t);
      gy += __shfl_sync(kFull, ay, t);
      gz += __shfl_sync(kFull, az, t);
      gn2 += __shfl_sync(kFull, an, t);
    }
  });
  if (lane == 0) {
    const float rest = s.rest;
    const float constraint = fmaxf(density, 1e-6f) / rest - 1.0f;
    const float denom = (gx * gx + gy * gy + gz * gz + gn2) / (rest * rest) + s.eps;
    lam[i] = make_float2(fmaxf(density, 1e-6f), -constraint / fmaxf(denom, 1e-9f));
    sq[i] = make_float4(gx, gy, gz, gn2);
  }
}

// sph_delta.glsl:19-85 + sph_apply_delta.glsl:10-20
__global__ void __launch_bounds__(kBlock) k_ad_delta_apply(const SegParams *__restrict__ segs, GridView g,
                                                           const float4 *__restrict__ pred,
                                                           const float2 *__restrict__ lam, int n,
                                                           float4 *__restrict__ out)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float4 pi = pred[i];
  const float lambda_i = lam[i].y;
  const float h = s.h, h2 = s.h2, spiky = s.spiky, poly6 = s.poly6, scorr_k = s.scorr_k, w_q = s.w_q;
  const bool use_scorr = scorr_k > 0.0f && w_q > 1e-9f;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  warp_chunks<1>(s, g, cell_coord(s, pi.x, pi.y, pi.z), lane, [&](bool valid, int j) {
    float tx = 0.0f, ty = 0.0f, tz = 0.0f;
    bool take = false;
    if (valid && j != i) {
      const float4 pj = __ldg(&pred[j]);
      const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < h2 && r2 > 1e-12f) {
        const float r = sqrtf(r2);
        const float lambda_j = __ldg(&lam[j].y);
        float s_corr = 0.0f;
        if (use_scorr) {
          const float ratio = w_poly6(r2, h2, poly6) / w_q;
          const float rr = fmaxf(ratio, 0.0f);
          const float rr2 = rr * rr;
          s_corr = -scorr_k * (rr2 * rr2);
        }
        const float sc = (lambda_i + lambda_j + s_corr) * w_spiky_grad(r, h, spiky);
        tx = sc * (dx / r);
        ty = sc * (dy / r);
        tz = sc * (dz / r);
        take = true;
      }
    }
    unsigned m = __ballot_sync(kFull, take);
    while (m) {
      const int t = __ffs(m) - 1;
      m &= m - 1;
      ax += __shfl_sync(kFull, tx, t);
      ay += __shfl_sync(kFull, ty, t);
      az += __shfl_sync(kFull, tz, t);
    }
  });
  if (lane == 0) {
    const float rest = s.rest;
    out[i] = make_float4(pi.x + ax / rest, pi.y + ay / rest, pi.z + az / rest, 1.0f);
  }
}

// sph_velocity.glsl + sph_xsph.glsl + sph_finalize.glsl. Keeps the velocity
// pass's v and the XSPH result v + dv for the adjoint, and the state the next
// substep starts from.
__global__ void __launch_bounds__(kBlock) k_ad_final(const SegParams *__restrict__ segs, GridView g,
                                                     const float4 *__restrict__ pred,
                                                     const float4 *__restrict__ pos,
                                                     const float2 *__restrict__ lam,
                                                     const uint8_t *__restrict__ collider, int n,
                                                     float4 *__restrict__ v_out, float4 *__restrict__ vf_out,
                                                     float4 *__restrict__ pos_next, float4 *__restrict__ vel_next,
                                                     float4 *__restrict__ pred_next, float *__restrict__ rho_next)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float dtc = s.dtc, h2 = s.h2, mass = s.mass, poly6 = s.poly6;
  const float4 q = pred[i];
  const float4 p0 = pos[i];
  const float3 vi = make_float3((q.x - p0.x) / dtc, (q.y - p0.y) / dtc, (q.z - p0.z) / dtc);
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  warp_chunks<1>(s, g, cell_coord(s, q.x, q.y, q.z), lane, [&](bool valid, int j) {
    float tx = 0.0f, ty = 0.0f, tz = 0.0f;
    bool take = false;
    if (valid && j != i) {
      const float4 pj = __ldg(&pred[j]);
      const float dx = q.x - pj.x, dy = q.y - pj.y, dz = q.z - pj.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < h2) {
        const float rho_j = fmaxf(__ldg(&lam[j].x), 1e-6f);
        const float4 xj = __ldg(&pos[j]);
        const float vjx = (pj.x - xj.x) / dtc, vjy = (pj.y - xj.y) / dtc, vjz = (pj.z - xj.z) / dtc;
        const float w = mass / rho_j;
        const float wk = w_poly6(r2, h2, poly6);
        tx = (w * (vjx - vi.x)) * wk;
        ty = (w * (vjy - vi.y)) * wk;
        tz = (w * (vjz - vi.z)) * wk;
        take = true;
      }
    }
    unsigned m = __ballot_sync(kFull, take);
    while (m) {
      const int t = __ffs(m) - 1;
      m &= m - 1;
      ax += __shfl_sync(kFull, tx, t);
      ay += __shfl_sync(kFull, ty, t);
      az += __shfl_sync(kFull, tz, t);
    }
  });
  if (lane != 0) return;
  const float c = s.visc;
  float3 v = make_float3(vi.x + c * ax, vi.y + c * ay, vi.z + c * az);
  v_out[i] = make_float4(vi.x, vi.y, vi.z, 0.0f);
  vf_out[i] = make_float4(v.x, v.y, v.z, 0.0f);
  float3 p = make_float3(q.x, q.y, q.z);
  finalize_particle(s, collider, p, v);
  pos_next[i] = make_float4(p.x, p.y, p.z, 1.0f);
  vel_next[i] = make_float4(v.x, v.y, v.z, 0.0f);
  pred_next[i] = q;
  rho_next[i] = lam[i].x;
}

// surface_splat.glsl:32-97 over the last grid, positions in id order.
__global__ void __launch_bounds__(kBlock) k_ad_splat(const SegParams *__restrict__ segs, GridView g, SplatGeom sp,
                                                     const float4 *__restrict__ pos,
                                                     const uint8_t *__restrict__ collider, long long samples,
                                                     float *__restrict__ out)
{
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= samples) return;
  const SegParams &s = segs[0];
  const int gx = (int)(t % sp.snx);
  const int gy = (int)((t / sp.snx) % sp.sny);
  const int gz = (int)(t / ((long long)sp.snx * sp.sny));
  const float px = sp.slox + (float)gx * sp.spacing;
  const float py = sp.sloy + (float)gy * sp.spacing;
  const float pz = sp.sloz + (float)gz * sp.spacing;
  float density = 0.0f;
  for_each_id<kSurfaceCellRadius>(s, g, cell_coord(s, px, py, pz), [&](int j) {
    const float4 pj = __ldg(&pos[j]);
    const float dx = px - pj.x, dy = py - pj.y, dz = pz - pj.z;
    density += sp.mass * w_poly6(dx * dx + dy * dy + dz * dz, sp.kh2, sp.kcoef);
  });
  float value = density / fmaxf(sp.rest, 1e-6f);
  if (s.voxel > 0.0f) {
    const int3 c = collider_coord(s, px, py, pz);
    if (collider_occupied(s, collider, c.x, c.y, c.z)) value = 0.0f;
  }
  out[t] = value;
}

// Grid bookkeeping after a counting-sort build: sorted ids, each particle's
// slot, and (copied from the key scratch) each particle's cell.
__global__ void k_ad_store_grid(const unsigned long long *__restrict__ pairs, const uint32_t *__restrict__ key_tmp,
                                int n, uint32_t *__restrict__ ids, uint32_t *__restrict__ slot,
                                uint32_t *__restrict__ cell)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t id = (uint32_t)(pairs[k] >> 32);
  ids[k] = id;
  slot[id] = (uint32_t)k;
  cell[k] = key_tmp[k];  // the key pass ran on identity slots: key_tmp[id]
}

__global__ void k_iota_u32(uint32_t *__restrict__ a, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) a[k] = (uint32_t)k;
}

// ---- reverse passes ----------------------------------------------------------

// Finalize (sph_finalize.glsl:13-96) replayed for particle i, then reversed:
// cotangents (gp, gv) of the finalized (position, velocity) to those of the
// predicted position (gp_in) and of the XSPH velocity (gvf).
__device__ void finalize_adjoint(const SegParams &s, const uint8_t *__restrict__ col, float3 p, float3 vf, float3 gp,
                                 float3 gv, float3 &gp_in, float3 &gvf)
{
  bool hit = false, vneg = false;
  float dist = 0.0f;
  float3 u = make_float3(0.f, 0.f, 1.f);
  float3 v = vf;
  const float voxel = s.voxel;
  if (voxel > 0.0f) {
    const int3 c = collider_coord(s, p.x, p.y, p.z);
    if (collider_occupied(s, col, c.x, c.y, c.z)) {
      float bx = 0.0f, by = 0.0f, bz = 0.0f, best = 1e30f;
      bool found = false;
      for (int dz = -kMaxColliderSearch; dz <= kMaxColliderSearch; ++dz)
        for (int dy = -kMaxColliderSearch; dy <= kMaxColliderSearch; ++dy)
          for (int dx = -kMaxColliderSearch; dx <= kMaxColliderSearch; ++dx) {
            const int nx = c.x + dx, ny = c.y + dy, nz = c.z + dz;
            if (nx < 0 || ny < 0 || nz < 0 || nx >= s.col_nx || ny >= s.col_ny || nz >= s.col_nz) continue;
            if (collider_occupied(s, col, nx, ny, nz)) continue;
            const float cx = s.lox + ((float)nx + 0.5f) * voxel;
            const float cy = s.loy + ((float)ny + 0.5f) * voxel;
            const float cz = s.loz + ((float)nz + 0.5f) * voxel;
            const float ex = cx - p.x, ey = cy - p.y, ez = cz - p.z;
            const float d2 = ex * ex + ey * ey + ez * ez;
            if (d2 < best) {
              best = d2;
              bx = cx;
              by = cy;
              bz = cz;
              found = true;
            }
          }
      if (found) {
        hit = true;
        dist = sqrtf(best);
        if (dist > 1e-6f) u = make_float3((bx - p.x) / dist, (by - p.y) / dist, (bz - p.z) / dist);
        const float push = dist + s.radius;
        p = make_float3(p.x + u.x * push, p.y + u.y * push, p.z + u.z * push);
        const float vn = v.x * u.x + v.y * u.y + v.z * u.z;
        if (vn < 0.0f) vneg = true;
      }
    }
  }
  // box clamp: a clamped axis forgets the position, reflects the velocity
  const float r = s.radius, damp = s.damping;
  const float lo[3] = {s.lox + r, s.loy + r, s.loz + r}, hi[3] = {s.hix - r, s.hiy - r, s.hiz - r};
  const float pa[3] = {p.x, p.y, p.z};
  float g1p[3] = {gp.x, gp.y, gp.z}, g1v[3] = {gv.x, gv.y, gv.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (pa[a] < lo[a] || pa[a] > hi[a]) {
      g1p[a] = 0.0f;
      g1v[a] = -damp * g1v[a];
    }
  }
  const float3 gp1 = make_float3(g1p[0], g1p[1], g1p[2]);
  const float3 gv1 = make_float3(g1v[0], g1v[1], g1v[2]);
  if (!hit) {
    gp_in = gp1;
    gvf = gv1;
    return;
  }
  gvf = gv1;
  float3 gu = make_float3(0.f, 0.f, 0.f);
  if (vneg) {
    // v1 = vf - (1 + damping) (vf . u) u
    const float ud = dot3(u, gv1);
    gvf = sub3(gv1, scale3(u, (1.0f + damp) * ud));
    gu = scale3(add3(scale3(gv1, dot3(vf, u)), scale3(vf, ud)), -(1.0f + damp));
  }
  if (dist > 1e-6f) {
    // p1 = best + radius u, u = (best - p) / |best - p|
    const float3 gg = add3(scale3(gp1, s.radius), gu);
    gp_in = scale3(sub3(gg, scale3(u, dot3(u, gg))), -1.0f / dist);
  } else {
    gp_in = gp1;  // u is the fixed fallback direction
  }
}

// Finalize reverse: seeds the cotangent of the last iterate (plus what the
// next substep's normal pass sent to it) and of the XSPH velocity.
__global__ void __launch_bounds__(kBlock) k_rv_final(const SegParams *__restrict__ segs,
                                                     const float4 *__restrict__ pred,
                                                     const float4 *__restrict__ vf,
                                                     const uint8_t *__restrict__ collider,
                                                     const float4 *__restrict__ g_pos_out,
                                                     const float4 *__restrict__ g_vel_out,
                                                     const float4 *__restrict__ g_pred_out, int n,
                                                     float4 *__restrict__ g_p, float4 *__restrict__ g_vf)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 gp_in, gvf;
  finalize_adjoint(segs[0], collider, f3(pred[i]), f3(vf[i]), f3(g_pos_out[i]), f3(g_vel_out[i]), gp_in, gvf);
  g_vf[i] = make_float4(gvf.x, gvf.y, gvf.z, 0.0f);
  const float4 go = g_pred_out[i];
  g_p[i] = make_float4(go.x + gp_in.x, go.y + gp_in.y, go.z + gp_in.z, 0.0f);
}

// XSPH reverse: dv_i = c sum_j (m / rho_j)(v_j - v_i) W(r_ij).
__global__ void __launch_bounds__(kBlock) k_rv_xsph(const SegParams *__restrict__ segs, GridView g,
                                                    const float4 *__restrict__ pred,
                                                    const float4 *__restrict__ v,
                                                    const float2 *__restrict__ lam,
                                                    const float4 *__restrict__ g_vf, int n,
                                                    float4 *__restrict__ g_v, float4 *__restrict__ g_p,
                                                    float *__restrict__ g_rho)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float h2 = s.h2, mass = s.mass, poly6 = s.poly6, c = s.visc;
  const float4 q = pred[i];
  const float3 vi = f3(v[i]);
  const float3 gvf = f3(g_vf[i]);
  float3 acc_v = make_float3(0.f, 0.f, 0.f), acc_p = make_float3(0.f, 0.f, 0.f);
  warp_chunks<1>(s, g, cell_coord(s, q.x, q.y, q.z), lane, [&](bool valid, int j) {
    if (!valid || j == i) return;
    const float4 pj = __ldg(&pred[j]);
    const float3 d = make_float3(q.x - pj.x, q.y - pj.y, q.z - pj.z);
    const float r2 = dot3(d, d);
    if (r2 >= h2) return;
    const float rho_j = fmaxf(__ldg(&lam[j].x), 1e-6f);
    const float w = mass / rho_j;
    const float t = h2 - r2;
    const float wk = poly6 * t * t * t;
    const float3 dv = sub3(f3(__ldg(&v[j])), vi);
    const float coef = c * w * wk;
    acc_v = sub3(acc_v, scale3(gvf, coef));
    atomic_add3(&g_v[j], scale3(gvf, coef));
    const float e = c * w * dot3(dv, gvf);
    const float3 dd = scale3(d, e * -6.0f * poly6 * t * t);  // e dW/dd
    acc_p = add3(acc_p, dd);
    atomic_add3(&g_p[j], scale3(dd, -1.0f));
    atomicAdd(&g_rho[j], -c * (mass / (rho_j * rho_j)) * dot3(dv, gvf) * wk);
  });
  acc_v = make_float3(warp_sum(acc_v.x), warp_sum(acc_v.y), warp_sum(acc_v.z));
  acc_p = make_float3(warp_sum(acc_p.x), warp_sum(acc_p.y), warp_sum(acc_p.z));
  if (lane == 0) {
    atomic_add3(&g_v[i], add3(gvf, acc_v));
    atomic_add3(&g_p[i], acc_p);
  }
}

// Velocity reverse: v = (p - x) / dt.
__global__ void k_rv_velocity(const SegParams *__restrict__ segs, const float4 *__restrict__ g_v, int n,
                              float4 *__restrict__ g_p, float4 *__restrict__ g_pos)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float inv = 1.0f / segs[0].dtc;
  const float4 gv = g_v[i];
  float4 gp = g_p[i];
  gp.x += gv.x * inv;
  gp.y += gv.y * inv;
  gp.z += gv.z * inv;
  g_p[i] = gp;
  g_pos[i] = make_float4(-gv.x * inv, -gv.y * inv, -gv.z * inv, 0.0f);
}

// Delta + apply reverse for one Jacobi iteration: p' = p + (1/rho0) sum_j
// (lambda_i + lambda_j + s_corr(r)) spiky (h - r)^2 d / r. Accumulates the
// cotangent of p (identity part included) and of lambda.
__global__ void __launch_bounds__(kBlock) k_rv_delta(const SegParams *__restrict__ segs, GridView g,
                                                     const float4 *__restrict__ pred,
                                                     const float2 *__restrict__ lam,
                                                     const float4 *__restrict__ g_next, int n,
                                                     float4 *__restrict__ g_cur, float *__restrict__ g_lam)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float h = s.h, h2 = s.h2, spiky = s.spiky, poly6 = s.poly6, scorr_k = s.scorr_k, w_q = s.w_q;
  const bool use_scorr = scorr_k > 0.0f && w_q > 1e-9f;
  const float4 pi = pred[i];
  const float lambda_i = lam[i].y;
  const float3 gn = f3(g_next[i]);
  const float3 a = scale3(gn, 1.0f / s.rest);
  float3 acc_p = make_float3(0.f, 0.f, 0.f);
  float acc_l = 0.0f;
  warp_chunks<1>(s, g, cell_coord(s, pi.x, pi.y, pi.z), lane, [&](bool valid, int j) {
    if (!valid || j == i) return;
    const float4 pj = __ldg(&pred[j]);
    const float3 d = make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
    const float r2 = dot3(d, d);
    if (r2 >= h2 || r2 <= 1e-12f) return;
    const float r = sqrtf(r2);
    const float hr = h - r;
    const float3 G = scale3(d, spiky * hr * hr / r);
    const float gdot = dot3(G, a);
    acc_l += gdot;
    atomicAdd(&g_lam[j], gdot);
    float cij = lambda_i + __ldg(&lam[j].y);
    float3 dd = make_float3(0.f, 0.f, 0.f);
    if (use_scorr) {
      const float t = h2 - r2;
      const float ratio = poly6 * t * t * t / w_q;
      const float rr2 = ratio * ratio;
      cij += -scorr_k * (rr2 * rr2);
      // d s_corr / dd = -4 k ratio^3 / w_q * (-6 poly6 t^2 d)
      dd = scale3(d, gdot * 24.0f * scorr_k * ratio * rr2 / w_q * poly6 * t * t);
    }
    dd = add3(dd, scale3(jphi(d, r, h, a), cij * spiky));
    acc_p = add3(acc_p, dd);
    atomic_add3(&g_cur[j], scale3(dd, -1.0f));
  });
  acc_p = make_float3(warp_sum(acc_p.x), warp_sum(acc_p.y), warp_sum(acc_p.z));
  acc_l = warp_sum(acc_l);
  if (lane == 0) {
    atomic_add3(&g_cur[i], add3(gn, acc_p));
    atomicAdd(&g_lam[i], acc_l);
  }
}

// Lambda reverse: lambda = -C / max(denom, 1e-9), C = max(rho, 1e-6) / rho0 - 1,
// denom = (|sum g|^2 + sum |g|^2) / rho0^2 + eps, rho = sum m W. g_rho_ext is
// the cotangent of the stored density max(rho, 1e-6) from its other users
// (XSPH and the next substep's normal pass), or NULL.
__global__ void __launch_bounds__(kBlock) k_rv_lambda(const SegParams *__restrict__ segs, GridView g,
                                                      const float4 *__restrict__ pred,
                                                      const float2 *__restrict__ lam,
                                                      const float4 *__restrict__ sq,
                                                      const float *__restrict__ g_lam,
                                                      const float *__restrict__ g_rho_ext, int n,
                                                      float4 *__restrict__ g_cur)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float h = s.h, h2 = s.h2, mass = s.mass, poly6 = s.poly6, spiky = s.spiky, rest = s.rest;
  const float2 li = lam[i];
  const float4 sqi = sq[i];
  const float3 S = f3(sqi);
  const float C = li.x / rest - 1.0f;
  const float denom = (dot3(S, S) + sqi.w) / (rest * rest) + s.eps;
  const float D = fmaxf(denom, 1e-9f);
  const float gl = g_lam[i];
  const float gC = -gl / D;
  const float gD = denom > 1e-9f ? gl * C / (D * D) : 0.0f;
  float grho = gC / rest + (g_rho_ext ? g_rho_ext[i] : 0.0f);
  if (!(li.x > 1e-6f)) grho = 0.0f;  // density clamped at 1e-6
  const float3 gS = scale3(S, 2.0f * gD / (rest * rest));
  const float gQ = gD / (rest * rest);
  if (grho == 0.0f && gD == 0.0f) return;  // uniform across the warp
  const float4 pi = pred[i];
  float3 acc = make_float3(0.f, 0.f, 0.f);
  warp_chunks<1>(s, g, cell_coord(s, pi.x, pi.y, pi.z), lane, [&](bool valid, int j) {
    if (!valid || j == i) return;
    const float4 pj = __ldg(&pred[j]);
    const float3 d = make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
    const float r2 = dot3(d, d);
    if (r2 >= h2) return;
    const float t = h2 - r2;
    float3 dd = scale3(d, grho * mass * -6.0f * poly6 * t * t);
    if (r2 > 1e-12f) {
      const float r = sqrtf(r2);
      const float hr = h - r;
      const float3 gij = scale3(d, mass * spiky * hr * hr / r);
      const float3 gbar = add3(gS, scale3(gij, 2.0f * gQ));
      dd = add3(dd, scale3(jphi(d, r, h, gbar), mass * spiky));
    }
    acc = add3(acc, dd);
    atomic_add3(&g_cur[j], scale3(dd, -1.0f));
  });
  acc = make_float3(warp_sum(acc.x), warp_sum(acc.y), warp_sum(acc.z));
  if (lane == 0) atomic_add3(&g_cur[i], acc);
}

// Predict reverse (sph_predict.glsl:23-57) with the normal pass's curvature
// (curv = -lap / |n|) folded in: cotangents of the position and velocity
// entering the substep, and of the normal pass's (n, lap).
__global__ void __launch_bounds__(kBlock) k_rv_predict(const SegParams *__restrict__ segs,
                                                       const float4 *__restrict__ vel,
                                                       const float4 *__restrict__ normal,
                                                       const float4 *__restrict__ g_q, int n,
                                                       float4 *__restrict__ g_pos, float4 *__restrict__ g_vel,
                                                       float4 *__restrict__ g_normal)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SegParams &s = segs[0];
  const float dt = s.dt;
  const float3 gq = f3(g_q[i]);
  float4 gpos = g_pos[i];
  g_pos[i] = make_float4(gpos.x + gq.x, gpos.y + gq.y, gpos.z + gq.z, 0.0f);
  // replay the velocity before the clamp
  const float4 v4 = vel[i];
  float3 v0 = make_float3(v4.x, v4.y, v4.z + s.gravity * dt);
  float4 nn = make_float4(0.f, 0.f, 0.f, 0.f);
  float mag = 0.0f;
  bool coh = false;
  if (s.sigma > 0.0f) {
    nn = normal[i];
    mag = sqrtf(nn.x * nn.x + nn.y * nn.y + nn.z * nn.z);
    if (mag > 1e-4f) {
      coh = true;
      const float sc = -s.sigma * nn.w;
      v0.x += ((sc * nn.x) / mag / s.mass) * dt;
      v0.y += ((sc * nn.y) / mag / s.mass) * dt;
      v0.z += ((sc * nn.z) / mag / s.mass) * dt;
    }
  }
  float3 gv = scale3(gq, dt);
  const float speed = sqrtf(dot3(v0, v0));
  if (speed > s.v_max) {
    const float3 uh = scale3(v0, 1.0f / speed);
    gv = scale3(sub3(gv, scale3(uh, dot3(uh, gv))), s.v_max / speed);
  }
  g_vel[i] = make_float4(gv.x, gv.y, gv.z, 0.0f);
  if (!coh) {
    g_normal[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float3 nv = make_float3(nn.x, nn.y, nn.z);
  const float sc = -s.sigma * nn.w;
  const float ndg = dot3(nv, gv);
  const float gcurv = -s.sigma * dt / (mag * s.mass) * ndg;
  float3 gnv = scale3(sub3(scale3(gv, 1.0f / mag), scale3(nv, ndg / (mag * mag * mag))), sc * dt / s.mass);
  // curv = -lap / mag
  const float lap = -nn.w * mag;
  const float glap = -gcurv / mag;
  gnv = add3(gnv, scale3(nv, gcurv * lap / (mag * mag * mag)));
  g_normal[i] = make_float4(gnv.x, gnv.y, gnv.z, glap);
}

// Normal reverse over the previous substep's grid: n_i = sum w_j poly6' (h^2 -
// r^2)^2 d, lap_i = sum w_j vlap (h - r), w_j = m / max(rho_j, 1e-6).
__global__ void __launch_bounds__(kBlock) k_rv_normal(const SegParams *__restrict__ segs, GridView g,
                                                      const float4 *__restrict__ pred,
                                                      const float *__restrict__ rho,
                                                      const float4 *__restrict__ g_normal, int n,
                                                      float4 *__restrict__ g_pred, float *__restrict__ g_rho)
{
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const float4 gn4 = g_normal[i];
  if (gn4.x == 0.0f && gn4.y == 0.0f && gn4.z == 0.0f && gn4.w == 0.0f) return;  // uniform across the warp
  const SegParams &s = segs[0];
  const float h = s.h, h2 = s.h2, mass = s.mass, poly6m6 = s.poly6m6, vlap = s.visclap;
  const float3 gn = f3(gn4);
  const float glap = gn4.w;
  const float4 pi = pred[i];
  float3 acc = make_float3(0.f, 0.f, 0.f);
  warp_chunks<1>(s, g, cell_coord(s, pi.x, pi.y, pi.z), lane, [&](bool valid, int j) {
    if (!valid || j == i) return;
    const float4 pj = __ldg(&pred[j]);
    const float3 d = make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
    const float r2 = dot3(d, d);
    if (r2 >= h2) return;
    const float rj = __ldg(&rho[j]);
    const float rho_j = fmaxf(rj, 1e-6f);
    const float w = mass / rho_j;
    const float t = h2 - r2;
    const float r = sqrtf(r2);
    float3 dd = scale3(sub3(scale3(gn, t * t), scale3(d, 4.0f * t * dot3(d, gn))), w * poly6m6);
    if (r > 0.0f) dd = sub3(dd, scale3(d, w * vlap * glap / r));
    acc = add3(acc, dd);
    atomic_add3(&g_pred[j], scale3(dd, -1.0f));
    if (rj > 1e-6f)
      atomicAdd(&g_rho[j], -(mass / (rho_j * rho_j)) * (poly6m6 * t * t * dot3(d, gn) + vlap * (h - r) * glap));
  });
  acc = make_float3(warp_sum(acc.x), warp_sum(acc.y), warp_sum(acc.z));
  if (lane == 0) atomic_add3(&g_pred[i], acc);
}

// Splat reverse, gathered per particle (one warp, lanes over the samples its
// kernel reaches): value(x) = sum_j m W(|x - p_j|^2) / rho0 over the
// candidates of x's cells.
__global__ void __launch_bounds__(kBlock) k_rv_splat(const SegParams *__restrict__ segs, GridView g, SplatGeom sp,
                                                     const float4 *__restrict__ pos,
                                                     const uint8_t *__restrict__ collider,
                                                     const float *__restrict__ g_surface, int n,
                                                     float4 *__restrict__ g_pos)
{
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  const SegParams &s = segs[0];
  const float4 pj = pos[j];
  const uint32_t cj = g.cell[j];
  const int cjx = (int)(cj % (uint32_t)s.nx), cjy = (int)((cj / (uint32_t)s.nx) % (uint32_t)s.ny),
            cjz = (int)(cj / ((uint32_t)s.nx * (uint32_t)s.ny));
  if (g.slot[j] >= __ldg(&g.off[cj]) + (uint32_t)kMaxCellScan) return;  // beyond the per-cell scan limit
  const float scale = sp.mass / fmaxf(sp.rest, 1e-6f) * 6.0f * sp.kcoef;
  int lo[3], ext[3];
  const float pc[3] = {pj.x, pj.y, pj.z}, sl[3] = {sp.slox, sp.sloy, sp.sloz};
  const int dims[3] = {sp.snx, sp.sny, sp.snz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    lo[a] = max((int)floorf((pc[a] - sp.kr - sl[a]) / sp.spacing) - 1, 0);
    ext[a] = max(min((int)floorf((pc[a] + sp.kr - sl[a]) / sp.spacing) + 1, dims[a] - 1) - lo[a] + 1, 0);
  }
  const int total = ext[0] * ext[1] * ext[2];
  float3 acc = make_float3(0.f, 0.f, 0.f);
  for (int u = lane; u < total; u += 32) {
    const int gx = lo[0] + u % ext[0], gy = lo[1] + (u / ext[0]) % ext[1], gz = lo[2] + u / (ext[0] * ext[1]);
    const float px = sp.slox + (float)gx * sp.spacing;
    const float py = sp.sloy + (float)gy * sp.spacing;
    const float pz = sp.sloz + (float)gz * sp.spacing;
    const float dx = px - pj.x, dy = py - pj.y, dz = pz - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 >= sp.kh2) continue;
    const int3 b = cell_coord(s, px, py, pz);
    if (abs(b.x - cjx) > kSurfaceCellRadius || abs(b.y - cjy) > kSurfaceCellRadius ||
        abs(b.z - cjz) > kSurfaceCellRadius)
      continue;
    if (s.voxel > 0.0f) {
      const int3 c = collider_coord(s, px, py, pz);
      if (collider_occupied(s, collider, c.x, c.y, c.z)) continue;
    }
    const long long t = ((long long)gz * sp.sny + gy) * sp.snx + gx;
    const float tt = sp.kh2 - r2;
    const float k = g_surface[t] * scale * tt * tt;
    acc = add3(acc, make_float3(k * dx, k * dy, k * dz));
  }
  acc = make_float3(warp_sum(acc.x), warp_sum(acc.y), warp_sum(acc.z));
  if (lane == 0) {
    const float4 gp = g_pos[j];
    g_pos[j] = make_float4(gp.x + acc.x, gp.y + acc.y, gp.z + acc.z, 0.0f);
  }
}

__global__ void k_combine_initial(const float4 *__restrict__ g_pos, const float4 *__restrict__ g_pred,
                                  const float4 *__restrict__ g_vel, int n, float4 *__restrict__ out_pos,
                                  float4 *__restrict__ out_vel)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = g_pos[i], b = g_pred[i], v = g_vel[i];
  out_pos[i] = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, 0.0f);
  out_vel[i] = make_float4(v.x, v.y, v.z, 0.0f);
}

}  // namespace

// ---- host object -------------------------------------------------------------
struct Adjoint {
  int device = 0;
  cudaStream_t stream = nullptr;
  int n = 0, cap_cells = 0, max_substeps = 0, max_iterations = 0, sm_count = 0;
  long long cap_voxels = 0, cap_samples = 0;
  std::string err;
  std::vector<void *> owned;

  // last forward
  bool recorded = false, collider_installed = false, splat_on = false;
  int substeps = 0, iterations = 0, cells = 0;
  int col_dims[3] = {0, 0, 0};
  float col_voxel = 0.0f;
  SegParams seg{};
  SplatGeom sp{}, sp_captured{};
  SegParams *d_seg = nullptr;
  uint8_t *collider = nullptr;

  // grid-build scratch (grid.cu's counting sort)
  DeviceState d{};
  // per grid g = 0..S: sorted ids, slot of each id, cell of each slot, offsets
  uint32_t *grid_ids = nullptr, *grid_slot = nullptr, *grid_cell = nullptr, *grid_off = nullptr;
  // checkpoints s = 0..S: state entering substep s
  float4 *ck_pos = nullptr, *ck_vel = nullptr, *ck_pred = nullptr;
  float *ck_rho = nullptr;
  // recompute workspace
  float4 *w_normal = nullptr, *w_p = nullptr, *w_sq = nullptr, *w_v = nullptr, *w_vf = nullptr;
  float2 *w_lam = nullptr;
  // cotangents
  float4 *g_pos_out = nullptr, *g_vel_out = nullptr, *g_pred_out = nullptr;
  float4 *g_pos_in = nullptr, *g_vel_in = nullptr, *g_pred_in = nullptr;
  float *g_rho_out = nullptr, *g_rho_in = nullptr, *g_rho_t = nullptr, *g_lam = nullptr;
  float4 *g_pa = nullptr, *g_pb = nullptr, *g_v = nullptr, *g_vf = nullptr, *g_normal = nullptr;
  // fixed buffers the captured graphs read and write
  float *surface_buf = nullptr, *g_surface = nullptr;
  float4 *g_init_pos = nullptr, *g_init_vel = nullptr;

  // The reverse pass swaps the cotangent buffers substep by substep; every
  // adjoint starts from the allocation order so a captured graph replays the
  // same buffer sequence.
  struct CotangentSet {
    float4 *pos_out, *vel_out, *pred_out, *pos_in, *vel_in, *pred_in, *pa, *pb;
    float *rho_out, *rho_in;
  } canon{};

  // One graph per direction, captured for the current (substeps, iterations,
  // splat, push block) and dropped when any of them changes.
  cudaGraphExec_t fwd_exec = nullptr, bwd_exec = nullptr;
  long long fwd_kernels = 0, bwd_kernels = 0;

  int fail(int code, const std::string &m)
  {
    err = m;
    return code;
  }
  int cuda(cudaError_t e, const char *what)
  {
    if (e == cudaSuccess) return FLOWX_OK;
    return fail(FLOWX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
  template <class T>
  cudaError_t alloc(T **p, size_t count)
  {
    cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) owned.push_back((void *)*p);
    return e;
  }

  size_t N() const { return (size_t)n; }
  GridView grid(int gi) const
  {
    GridView v;
    v.ids = grid_ids + (size_t)gi * N();
    v.slot = grid_slot + (size_t)gi * N();
    v.cell = grid_cell + (size_t)gi * N();
    v.off = grid_off + (size_t)gi * ((size_t)cap_cells + 1);
    return v;
  }
  float4 *ckp(float4 *base, int s) const { return base + (size_t)s * N(); }
  float *ckr(int s) const { return ck_rho + (size_t)s * N(); }
  float4 *wp(int t) const { return w_p + (size_t)t * N(); }
  float2 *wl(int t) const { return w_lam + (size_t)t * N(); }
  float4 *wsq(int t) const { return w_sq + (size_t)t * N(); }

  int allocate()
  {
    const size_t nn = N(), S1 = (size_t)max_substeps + 1, I = (size_t)max_iterations, c1 = (size_t)cap_cells + 1;
    cudaError_t e = cudaSuccess;
#define A(ptr, count) \
  if (e == cudaSuccess) e = alloc(&(ptr), (count));
    A(d_seg, 1) A(collider, (size_t)std::max<long long>(cap_voxels, 1))
    A(d.counts, (size_t)cap_cells) A(d.offsets, c1) A(d.block_sums, (size_t)cap_cells / 2048 + 2)
    A(d.big_cells, c1) A(d.key_tmp, nn) A(d.rank_tmp, nn) A(d.ids, nn) A(d.pairs, nn) A(d.pairs_tmp, nn)
    A(grid_ids, S1 * nn) A(grid_slot, S1 * nn) A(grid_cell, S1 * nn) A(grid_off, S1 * c1)
    A(ck_pos, S1 * nn) A(ck_vel, S1 * nn) A(ck_pred, S1 * nn) A(ck_rho, S1 * nn)
    A(w_normal, nn) A(w_p, (I + 1) * nn) A(w_sq, I * nn) A(w_lam, I * nn) A(w_v, nn) A(w_vf, nn)
    A(g_pos_out, nn) A(g_vel_out, nn) A(g_pred_out, nn) A(g_pos_in, nn) A(g_vel_in, nn) A(g_pred_in, nn)
    A(g_rho_out, nn) A(g_rho_in, nn) A(g_rho_t, nn) A(g_lam, nn) A(g_pa, nn) A(g_pb, nn) A(g_v, nn)
    A(g_vf, nn) A(g_normal, nn) A(surface_buf, (size_t)cap_samples) A(g_surface, (size_t)cap_samples)
    A(g_init_pos, nn) A(g_init_vel, nn)
#undef A
    if (e != cudaSuccess) return cuda(e, "adjoint allocation");
    canon = CotangentSet{g_pos_out, g_vel_out, g_pred_out, g_pos_in, g_vel_in, g_pred_in, g_pa, g_pb, g_rho_out,
                         g_rho_in};
    if (e == cudaSuccess) e = cudaMemsetAsync(d.counts, 0, sizeof(uint32_t) * (size_t)cap_cells, stream);
    if (e == cudaSuccess && n > 0) {
      k_iota_u32<<<blocks_for(n), kBlock, 0, stream>>>(d.ids, n);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return cuda(e, "adjoint initialisation");
  }

  void reset_cotangents()
  {
    g_pos_out = canon.pos_out;
    g_vel_out = canon.vel_out;
    g_pred_out = canon.pred_out;
    g_pos_in = canon.pos_in;
    g_vel_in = canon.vel_in;
    g_pred_in = canon.pred_in;
    g_pa = canon.pa;
    g_pb = canon.pb;
    g_rho_out = canon.rho_out;
    g_rho_in = canon.rho_in;
  }

  void drop_graphs()
  {
    if (fwd_exec) cudaGraphExecDestroy(fwd_exec);
    if (bwd_exec) cudaGraphExecDestroy(bwd_exec);
    fwd_exec = bwd_exec = nullptr;
  }

  // Capture `issue` on the stream into *exec (kernels counted into *kernels).
  template <class F>
  int capture(cudaGraphExec_t *exec, long long *kernels, F &&issue)
  {
    int rc = cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
    if (rc) return rc;
    const long long before = g_launches.load();
    issue();
    *kernels = g_launches.load() - before;
    g_launches -= *kernels;  // captured, not launched
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    return cuda(e, "graph capture");
  }

  void release()
  {
    drop_graphs();
    for (void *p : owned) cudaFree(p);
    owned.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }

  // Counting-sort build of grid gi from positions q (id order).
  void build_grid(int gi, const float4 *q)
  {
    d.segs = d_seg;
    d.nseg = 1;
    d.seg0 = seg;
    d.cseg_base = -1;
    d.n = n;
    d.cells = cells;
    d.sm_count = sm_count;
    launch_key_only(d, q, stream);
    launch_scan(d, stream);
    launch_scatter(d, stream);
    launch_cell_sort(d, stream);
    GridView g = grid(gi);
    if (n > 0)
      k_ad_store_grid<<<blocks_for(n), kBlock, 0, stream>>>(d.pairs, d.key_tmp, n, (uint32_t *)g.ids,
                                                            (uint32_t *)g.slot, (uint32_t *)g.cell);
    cudaMemcpyAsync((void *)g.off, d.offsets, sizeof(uint32_t) * ((size_t)cells + 1), cudaMemcpyDeviceToDevice,
                    stream);
    g_launches += 8;
  }

  // Substep s from checkpoint s: every iterate into the workspace, the
  // finalized state into checkpoint s + 1. build = build grid s + 1 (forward).
  void substep(int s, bool build)
  {
    const unsigned nb = blocks_for(n), nw = warp_blocks(n);
    if (seg.sigma > 0.0f) {
      k_ad_normal<<<nw, kBlock, 0, stream>>>(d_seg, grid(s), ckp(ck_pred, s), ckr(s), n, w_normal);
      g_launches += 1;
    }
    k_ad_predict<<<nb, kBlock, 0, stream>>>(d_seg, ckp(ck_pos, s), ckp(ck_vel, s), w_normal, n, wp(0));
    g_launches += 1;
    if (build) build_grid(s + 1, wp(0));
    const GridView g = grid(s + 1);
    for (int t = 0; t < iterations; ++t) {
      k_ad_lambda<<<nw, kBlock, 0, stream>>>(d_seg, g, wp(t), n, wl(t), wsq(t));
      k_ad_delta_apply<<<nw, kBlock, 0, stream>>>(d_seg, g, wp(t), wl(t), n, wp(t + 1));
    }
    k_ad_final<<<nw, kBlock, 0, stream>>>(d_seg, g, wp(iterations), ckp(ck_pos, s), wl(iterations - 1), collider, n,
                                          w_v, w_vf, ckp(ck_pos, s + 1), ckp(ck_vel, s + 1),
                                          ckp(ck_pred, s + 1), ckr(s + 1));
    g_launches += 2 * iterations + 2;
  }

  // Reverse of substep s (its recompute must be in the workspace). Reads the
  // cotangents of checkpoint s + 1 (g_*_out), writes those of checkpoint s
  // (g_*_in).
  void reverse(int s)
  {
    const unsigned nb = blocks_for(n), nw = warp_blocks(n);
    const size_t f4 = N() * sizeof(float4), f1 = N() * sizeof(float);
    const GridView g = grid(s + 1);
    cudaMemsetAsync(g_v, 0, f4, stream);
    cudaMemsetAsync(g_pred_in, 0, f4, stream);
    cudaMemsetAsync(g_rho_in, 0, f1, stream);
    cudaMemcpyAsync(g_rho_t, g_rho_out, f1, cudaMemcpyDeviceToDevice, stream);
    k_rv_final<<<nb, kBlock, 0, stream>>>(d_seg, wp(iterations), w_vf, collider, g_pos_out, g_vel_out, g_pred_out, n,
                                          g_pa, g_vf);
    k_rv_xsph<<<nw, kBlock, 0, stream>>>(d_seg, g, wp(iterations), w_v, wl(iterations - 1), g_vf, n, g_v, g_pa,
                                         g_rho_t);
    k_rv_velocity<<<nb, kBlock, 0, stream>>>(d_seg, g_v, n, g_pa, g_pos_in);
    g_launches += 3;
    for (int t = iterations - 1; t >= 0; --t) {
      cudaMemsetAsync(g_pb, 0, f4, stream);
      cudaMemsetAsync(g_lam, 0, f1, stream);
      k_rv_delta<<<nw, kBlock, 0, stream>>>(d_seg, g, wp(t), wl(t), g_pa, n, g_pb, g_lam);
      k_rv_lambda<<<nw, kBlock, 0, stream>>>(d_seg, g, wp(t), wl(t), wsq(t), g_lam,
                                             t == iterations - 1 ? g_rho_t : nullptr, n, g_pb);
      g_launches += 2;
      std::swap(g_pa, g_pb);
    }
    k_rv_predict<<<nb, kBlock, 0, stream>>>(d_seg, ckp(ck_vel, s), w_normal, g_pa, n, g_pos_in, g_vel_in, g_normal);
    g_launches += 1;
    if (seg.sigma > 0.0f) {
      k_rv_normal<<<nw, kBlock, 0, stream>>>(d_seg, grid(s), ckp(ck_pred, s), ckr(s), g_normal, n, g_pred_in,
                                             g_rho_in);
      g_launches += 1;
    }
    std::swap(g_pos_in, g_pos_out);
    std::swap(g_vel_in, g_vel_out);
    std::swap(g_pred_in, g_pred_out);
    std::swap(g_rho_in, g_rho_out);
  }
};

}  // namespace flowx

using namespace flowx;

namespace {
Adjoint *as_adj(flowx_adjoint *a) { return reinterpret_cast<Adjoint *>(a); }
thread_local std::string g_adjoint_create_error;
}  // namespace

extern "C" {

int flowx_adjoint_create(const flowx_adjoint_config *config, flowx_adjoint **out)
{
  if (!config || !out) {
    g_adjoint_create_error = "flowx_adjoint_create: config and out must not be NULL";
    return FLOWX_ERR_ARG;
  }
  *out = nullptr;
  const flowx_adjoint_config &c = *config;
  if (c.particle_count < 0 || c.max_cells < 1 || c.max_substeps < 1 || c.max_iterations < 1 ||
      c.max_iterations > kMaxIterations || c.max_collider_voxels < 0 || c.max_surface_samples < 0) {
    g_adjoint_create_error = "flowx_adjoint_create: need particle_count >= 0, max_cells, max_substeps >= 1, "
                             "1 <= max_iterations <= 1000, capacities >= 0";
    return FLOWX_ERR_ARG;
  }
  if (c.particle_count > (1 << 24)) {
    g_adjoint_create_error = "flowx_adjoint_create: particle_count above 2^24";
    return FLOWX_ERR_CAPACITY;
  }
  Adjoint *a = new Adjoint();
  a->device = c.device;
  a->n = c.particle_count;
  a->cap_cells = c.max_cells;
  a->max_substeps = c.max_substeps;
  a->max_iterations = c.max_iterations;
  a->cap_voxels = c.max_collider_voxels;
  a->cap_samples = c.max_surface_samples;
  int rc = a->cuda(cudaSetDevice(a->device), "cudaSetDevice");
  if (!rc) rc = a->cuda(cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking), "stream");
  if (!rc) rc = a->cuda(cudaDeviceGetAttribute(&a->sm_count, cudaDevAttrMultiProcessorCount, a->device), "attribute");
  if (!rc) rc = a->allocate();
  if (rc) {
    g_adjoint_create_error = a->err;
    a->release();
    delete a;
    return rc;
  }
  *out = reinterpret_cast<flowx_adjoint *>(a);
  return FLOWX_OK;
}

int flowx_adjoint_destroy(flowx_adjoint *adj)
{
  if (!adj) return FLOWX_OK;
  Adjoint *a = as_adj(adj);
  cudaSetDevice(a->device);
  if (a->stream) cudaStreamSynchronize(a->stream);
  a->release();
  delete a;
  return FLOWX_OK;
}

const char *flowx_adjoint_last_error(const flowx_adjoint *adj)
{
  if (!adj) return g_adjoint_create_error.c_str();
  return reinterpret_cast<const Adjoint *>(adj)->err.c_str();
}

int flowx_adjoint_get_stream(flowx_adjoint *adj, void **stream)
{
  if (!adj || !stream) return FLOWX_ERR_ARG;
  *stream = (void *)as_adj(adj)->stream;
  return FLOWX_OK;
}

int flowx_adjoint_set_collider(flowx_adjoint *adj, const uint8_t *occupancy, const int32_t dims[3], float voxel_size)
{
  if (!adj) return FLOWX_ERR_ARG;
  Adjoint *a = as_adj(adj);
  cudaSetDevice(a->device);
  if (!occupancy || !dims || !(voxel_size > 0.0f) || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
    return a->fail(FLOWX_ERR_ARG, "collider needs occupancy, positive dims and voxel size");
  const long long vox = (long long)dims[0] * dims[1] * dims[2];
  if (vox > a->cap_voxels) return a->fail(FLOWX_ERR_CAPACITY, "collider larger than max_collider_voxels");
  int rc = a->cuda(cudaMemcpyAsync(a->collider, occupancy, (size_t)vox, cudaMemcpyHostToDevice, a->stream),
                   "collider upload");
  if (!rc) rc = a->cuda(cudaStreamSynchronize(a->stream), "collider upload");
  if (rc) return rc;
  std::memcpy(a->col_dims, dims, sizeof(a->col_dims));
  a->col_voxel = voxel_size;
  a->collider_installed = true;
  return FLOWX_OK;
}

int flowx_adjoint_forward(flowx_adjoint *adj, const flowx_push *push, int iterations, int substeps,
                          const float *positions, const float *velocities, float *positions_out,
                          float *velocities_out, const flowx_push *splat_push, float *surface)
{
  if (!adj) return FLOWX_ERR_ARG;
  Adjoint *a = as_adj(adj);
  cudaSetDevice(a->device);
  a->recorded = false;
  if (!push || (a->n > 0 && (!positions || !velocities || !positions_out || !velocities_out)))
    return a->fail(FLOWX_ERR_ARG, "flowx_adjoint_forward: NULL push block or particle buffer");
  if (iterations < 1 || iterations > a->max_iterations)
    return a->fail(FLOWX_ERR_ARG, "iterations must be in [1, max_iterations]");
  if (substeps < 1 || substeps > a->max_substeps)
    return a->fail(FLOWX_ERR_ARG, "substeps must be in [1, max_substeps]");
  const long long cells = (long long)push->i_grid[0] * push->i_grid[1] * push->i_grid[2];
  if (push->i_layout[0] != a->n || push->i_grid[0] <= 0 || push->i_grid[1] <= 0 || push->i_grid[2] <= 0 ||
      cells != push->i_grid[3] || !(push->f_lo[3] > 0.0f))
    return a->fail(FLOWX_ERR_ARG, "push block: particle count or grid inconsistent with the object");
  if (cells > a->cap_cells) return a->fail(FLOWX_ERR_CAPACITY, "grid cells exceed max_cells");
  SegParams s{};
  seg_from_push(*push, s);
  s.p_begin = 0;
  s.c_begin = 0;
  s.col_begin = 0;
  if (s.voxel > 0.0f) {
    if (!a->collider_installed || a->col_dims[0] != s.col_nx || a->col_dims[1] != s.col_ny ||
        a->col_dims[2] != s.col_nz || a->col_voxel != s.voxel)
      return a->fail(FLOWX_ERR_STATE, "the push block names a collider that differs from the installed one");
  }
  if (splat_push) {
    const long long samples = (long long)splat_push->i_sort[0] * splat_push->i_sort[1] * splat_push->i_sort[2];
    if (!surface) return a->fail(FLOWX_ERR_ARG, "splat requested without a surface buffer");
    if (splat_push->i_sort[0] <= 0 || splat_push->i_sort[1] <= 0 || splat_push->i_sort[2] <= 0 ||
        samples > a->cap_samples)
      return a->fail(FLOWX_ERR_CAPACITY, "splat grid exceeds max_surface_samples");
    SplatGeom &sp = a->sp;
    sp.slox = splat_push->f_hi[0];
    sp.sloy = splat_push->f_hi[1];
    sp.sloz = splat_push->f_hi[2];
    sp.spacing = bits_to_float(splat_push->i_sort[3]);
    sp.kr = splat_push->f_sph[0];
    sp.kh2 = sp.kr * sp.kr;
    sp.kcoef = 315.0f / (64.0f * 3.14159265358979323846f * powf(sp.kr, 9.0f));
    sp.mass = splat_push->f_sph[1];
    sp.rest = splat_push->f_sph[2];
    sp.snx = splat_push->i_sort[0];
    sp.sny = splat_push->i_sort[1];
    sp.snz = splat_push->i_sort[2];
  }
  SplatGeom sp_new = a->sp;
  const bool splat_on = splat_push != nullptr;
  const bool same = a->fwd_exec && std::memcmp(&s, &a->seg, sizeof(SegParams)) == 0 && a->cells == (int)cells &&
                    a->iterations == iterations && a->substeps == substeps && a->splat_on == splat_on &&
                    (!splat_on || std::memcmp(&sp_new, &a->sp_captured, sizeof(SplatGeom)) == 0);
  cudaStream_t st = a->stream;
  int rc = FLOWX_OK;
  if (!same) {
    a->drop_graphs();
    a->seg = s;
    a->sp_captured = sp_new;
    a->cells = (int)cells;
    a->iterations = iterations;
    a->substeps = substeps;
    a->splat_on = splat_on;
    rc = a->cuda(cudaMemcpyAsync(a->d_seg, &a->seg, sizeof(SegParams), cudaMemcpyHostToDevice, st), "segment");
  }
  const long long samples = splat_on ? (long long)a->sp.snx * a->sp.sny * a->sp.snz : 0;
  const size_t f4 = a->N() * sizeof(float4);
  if (!rc && a->n > 0) {
    // initial state: predicted = positions, densities zero, grid from positions
    cudaMemcpyAsync(a->ckp(a->ck_pos, 0), positions, f4, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(a->ckp(a->ck_vel, 0), velocities, f4, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(a->ckp(a->ck_pred, 0), positions, f4, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(a->ckr(0), 0, a->N() * sizeof(float), st);
    if (!a->fwd_exec)
      rc = a->capture(&a->fwd_exec, &a->fwd_kernels, [&] {
        a->build_grid(0, a->ckp(a->ck_pos, 0));
        for (int sub = 0; sub < substeps; ++sub) a->substep(sub, true);
        if (splat_on) {
          k_ad_splat<<<blocks_for(samples), kBlock, 0, st>>>(a->d_seg, a->grid(substeps), a->sp,
                                                             a->ckp(a->ck_pos, substeps), a->collider, samples,
                                                             a->surface_buf);
          g_launches += 1;
        }
      });
    if (!rc) rc = a->cuda(cudaGraphLaunch(a->fwd_exec, st), "forward graph launch");
    if (!rc) g_launches += a->fwd_kernels;
    cudaMemcpyAsync(positions_out, a->ckp(a->ck_pos, substeps), f4, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(velocities_out, a->ckp(a->ck_vel, substeps), f4, cudaMemcpyDeviceToDevice, st);
    if (splat_on)
      cudaMemcpyAsync(surface, a->surface_buf, sizeof(float) * (size_t)samples, cudaMemcpyDeviceToDevice, st);
  } else if (!rc && splat_on) {
    cudaMemsetAsync(surface, 0, sizeof(float) * (size_t)samples, st);
  }
  if (!rc) rc = a->cuda(cudaGetLastError(), "flowx_adjoint_forward");
  if (!rc) a->recorded = true;
  return rc;
}

int flowx_substep_adjoint(flowx_adjoint *adj, const float *surface_grad, const float *positions_out_grad,
                          const float *velocities_out_grad, float *positions_grad, float *velocities_grad)
{
  if (!adj) return FLOWX_ERR_ARG;
  Adjoint *a = as_adj(adj);
  cudaSetDevice(a->device);
  if (!a->recorded) return a->fail(FLOWX_ERR_STATE, "flowx_substep_adjoint: no recorded forward");
  if (a->n > 0 && (!positions_grad || !velocities_grad))
    return a->fail(FLOWX_ERR_ARG, "flowx_substep_adjoint: gradient outputs are required");
  if (surface_grad && !a->splat_on)
    return a->fail(FLOWX_ERR_STATE, "surface cotangent given but the forward made no splat");
  if (a->n == 0) return FLOWX_OK;
  cudaStream_t st = a->stream;
  const size_t f4 = a->N() * sizeof(float4), f1 = a->N() * sizeof(float);
  const int S = a->substeps;
  const long long samples = a->splat_on ? (long long)a->sp.snx * a->sp.sny * a->sp.snz : 0;
  a->reset_cotangents();
  // cotangents of the final state into the buffers the graph reads
  if (positions_out_grad)
    cudaMemcpyAsync(a->g_pos_out, positions_out_grad, f4, cudaMemcpyDeviceToDevice, st);
  else
    cudaMemsetAsync(a->g_pos_out, 0, f4, st);
  if (velocities_out_grad)
    cudaMemcpyAsync(a->g_vel_out, velocities_out_grad, f4, cudaMemcpyDeviceToDevice, st);
  else
    cudaMemsetAsync(a->g_vel_out, 0, f4, st);
  if (a->splat_on) {
    if (surface_grad)
      cudaMemcpyAsync(a->g_surface, surface_grad, sizeof(float) * (size_t)samples, cudaMemcpyDeviceToDevice, st);
    else
      cudaMemsetAsync(a->g_surface, 0, sizeof(float) * (size_t)samples, st);
  }
  int rc = FLOWX_OK;
  if (!a->bwd_exec) {
    rc = a->capture(&a->bwd_exec, &a->bwd_kernels, [&] {
      cudaMemsetAsync(a->g_pred_out, 0, f4, st);
      cudaMemsetAsync(a->g_rho_out, 0, f1, st);
      if (a->splat_on) {
        k_rv_splat<<<warp_blocks(a->n), kBlock, 0, st>>>(a->d_seg, a->grid(S), a->sp, a->ckp(a->ck_pos, S),
                                                        a->collider, a->g_surface, a->n, a->g_pos_out);
        g_launches += 1;
      }
      for (int s = S - 1; s >= 0; --s) {
        a->substep(s, false);
        a->reverse(s);
      }
      // the first substep's predicted positions were the initial positions
      k_combine_initial<<<blocks_for(a->n), kBlock, 0, st>>>(a->g_pos_out, a->g_pred_out, a->g_vel_out, a->n,
                                                             a->g_init_pos, a->g_init_vel);
      g_launches += 1;
    });
    a->reset_cotangents();
  }
  if (!rc) rc = a->cuda(cudaGraphLaunch(a->bwd_exec, st), "adjoint graph launch");
  if (!rc) g_launches += a->bwd_kernels;
  cudaMemcpyAsync(positions_grad, a->g_init_pos, f4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(velocities_grad, a->g_init_vel, f4, cudaMemcpyDeviceToDevice, st);
  if (!rc) rc = a->cuda(cudaGetLastError(), "flowx_substep_adjoint");
  return rc;
}

}  // extern "C"
