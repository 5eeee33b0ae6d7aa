// PBF passes on the grid-ordered state: the fused substep kernels and the
// single reference passes (for the per-pass API), plus the per-frame density
// splat and the analytic collider voxeliser.
//
// Fused substep (solver/sph.py:501-514 as executed here):
//   normal          sph_normal.glsl                      (if sigma > 0)
//   predict_key     sph_predict.glsl + sph_grid_key.glsl (grid.cu)
//   scan/scatter/sort/permute                             (grid.cu)
//   I x { row_bounds  (the bounds lambda trims its rows with)
//         lambda    sph_lambda.glsl
//         delta_apply sph_delta.glsl + sph_apply_delta.glsl, written to the
//                     other predicted buffer (ping-pong) }
//   row_bounds
//   xsph_finalize   sph_velocity.glsl + sph_xsph.glsl + sph_finalize.glsl:
//                   neighbour velocities are re-derived from (pred - pos)/dt,
//                   the same expression sph_velocity.glsl stores, and the new
//                   positions go to the other position buffer so neighbours
//                   still read the old ones.
// Every neighbour pass uses the two-phase walk of neighbour.cuh.
#include "neighbour.cuh"

namespace flowx {

static inline int blk(const DeviceState &d, KernelId k, int def) { return d.block[k] > 0 ? d.block[k] : def; }
static inline unsigned grid_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

#define FLOWX_SLOT_PROLOGUE                            \
  const int i = blockIdx.x * blockDim.x + threadIdx.x; \
  if (i >= d.n) return;                                \
  const SegParams &s = d.segs[slot_segment(d, i)];

#define FLOWX_SLOT_PROLOGUE_SEG                        \
  const int i = blockIdx.x * blockDim.x + threadIdx.x; \
  if (i >= d.n) return;                                \
  const SegParams &s = slot_params<SEG>(d, i);

// ---- neighbour passes -------------------------------------------------------

// Register bounds of the neighbour kernels below, each measured on the
// 4M-particle workload: lambda and normal three 512-thread blocks per SM (at
// most 42 registers: the extra resident warps hide more of the candidate-load
// latency than the few registers cost, 1.6% per frame), delta_apply four
// (32), XSPH five 256-thread blocks (48).
// sph_lambda.glsl:17-77
template <bool EXACT, int SEG, bool TRIMMED>
__global__ void __launch_bounds__(512, 3) k_lambda_f(DeviceState d, const float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE_SEG
  const float4 pi = pred[i];
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  LambdaAcc<EXACT> acc;
  const MaskRecord rec{d.row_masks, d.row_wide, d.n, d.chunk_masks, d.chunk_base};
  const RowTrim trim{d.quad_bounds, d.row_yz};
  for_each_within_recording<EXACT, TRIMMED>(s, d.offsets, pred, d.quads, trim, pi, s.h2, base, rec, i, [&](int k, bool within) {
    const float4 pj = __ldg(&pred[k]);
    acc.pair(s, pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, within);
  });
  const float2 l = acc.finish(s);
  d.lam[i] = l;
  d.plam[i] = make_float4(pi.x, pi.y, pi.z, l.y);
}

// sph_delta.glsl:19-85, summed correction before the 1/rho0 scale. RECORDED:
// the lambda pass of this iteration just tested the same positions against
// the same grid with the same reach (r < h), so its recorded row masks stand
// in for phase 1; the body keeps its own j != i and r^2 > 1e-12 tests.
// RECORDED also reads each neighbour's position and lambda from d.plam (one
// 16-byte load; the lambda pass left them there).
template <bool EXACT, bool RECORDED, bool TRIMMED = false>
__device__ __forceinline__ float3 delta_sum_f(const SegParams &s, const DeviceState &d, const float4 *__restrict__ pred,
                                              int i, float4 pi)
{
  const float lambda_i = d.lam[i].y;
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  const float h2 = s.h2;
  auto body = [&](int k, bool within) {
    // j == i needs no test of its own: its r^2 is exactly 0, which the
    // r^2 <= 1e-12 test below rejects
    const float4 pj = RECORDED ? __ldg(&d.plam[k]) : __ldg(&pred[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = pair_r2<EXACT>(dx, dy, dz);
    if ((!within && r2 >= h2) || r2 <= 1e-12f) return;
    delta_pair<EXACT>(s, lambda_i, RECORDED ? pj.w : __ldg(&d.lam[k].y), dx, dy, dz, r2, ax, ay, az);
  };
  if (RECORDED)
    for_each_within_recorded<EXACT, TRIMMED>(s, d.offsets, pred, d.quads, RowTrim{d.quad_bounds, d.row_yz}, pi, h2,
                                         base, MaskRecord{d.row_masks, d.row_wide, d.n, d.chunk_masks, d.chunk_base}, i, body);
  else
    for_each_within<EXACT>(s, d.offsets, pred, pi, h2, base, body);
  return make_float3(ax, ay, az);
}

// sph_normal.glsl:56-74 for one neighbour: n = sum (m / rho_j) grad W_poly6
// and the curvature's laplacian sum. EXACT: the reference's operations; FAST:
// re-associated (FMA, one reciprocal square root).
template <bool EXACT>
__device__ __forceinline__ void normal_terms(const SegParams &s, float rho_j, float r2, float dx, float dy, float dz,
                                             float &nx, float &ny, float &nz, float &lap)
{
  if (EXACT) {
    const float weight = s.mass / rho_j;
    const float t = s.h2 - r2;
    const float sg = s.poly6m6 * t * t;
    nx += weight * (sg * dx);
    ny += weight * (sg * dy);
    nz += weight * (sg * dz);
    lap += weight * w_visc_lap(sqrtf(r2), s.h, s.visclap);
  } else {
    const float weight = __fdividef(s.mass, rho_j);
    const float t = __fsub_rn(s.h2, r2);
    const float sg = __fmul_rn(weight, __fmul_rn(s.poly6m6, __fmul_rn(t, t)));
    nx = __fmaf_rn(sg, dx, nx);
    ny = __fmaf_rn(sg, dy, ny);
    nz = __fmaf_rn(sg, dz, nz);
    // r = sqrt(r2); coincident particles (r2 = 0, e.g. two clamped into the
    // same box corner) have r = 0, as sqrtf gives.
    const float r = r2 > 0.0f ? __fmul_rn(r2, rsqrtf(r2)) : 0.0f;
    lap = __fmaf_rn(__fmul_rn(weight, s.visclap), __fsub_rn(s.h, r), lap);
  }
}

// sph_delta.glsl + sph_apply_delta.glsl: pred_out = pred_in + sum / rho0.
// last: also d.xv[i] for the XSPH pass that follows. The re-associated form
// is bounded to four 512-thread blocks per SM (32 registers, no spill): its
// gathers are latency-bound, and the full 64 resident warps hide more of them
// (0.726 -> 0.688 ms per launch on the 4M-particle workload); the reference
// form would spill at 32 and keeps three.
template <bool EXACT, int SEG, bool TRIMMED>
__global__ void __launch_bounds__(512, EXACT ? 3 : 4) k_delta_apply_f(DeviceState d, const float4 *__restrict__ pred_in,
                                                       float4 *__restrict__ pred_out, int last)
{
  FLOWX_SLOT_PROLOGUE_SEG
  const float4 pi = pred_in[i];
  const float3 a = delta_sum_f<EXACT, true, TRIMMED>(s, d, pred_in, i, pi);
  const float rest = s.rest;
  const float4 q = make_float4(pi.x + a.x / rest, pi.y + a.y / rest, pi.z + a.z / rest, 1.0f);
  pred_out[i] = q;
  store_quad(TRIMMED ? d.quads_alt : d.quads, i, q.x, q.y, q.z);
  if (last) d.xv[i] = xsph_input<EXACT>(s, d, i, q);
}

template <bool EXACT>
__global__ void k_xsph_inputs(DeviceState d, const float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE
  d.xv[i] = xsph_input<EXACT>(s, d, i, pred[i]);
}

__global__ void k_fill_quads(DeviceState d, const float4 *__restrict__ pred)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const float4 q = pred[i];
  store_quad(d.quads, i, q.x, q.y, q.z);
}

// The bounds the trimmed phase 1 of lambda and XSPH reads (RowTrim in
// neighbour.cuh), from the positions those passes test. One warp per x-row
// (the nx cells of one (y, z), whose slots are one contiguous run):
//  * per cell, the y and z bounds of the particles of its cells x - 1, x,
//    x + 1 (thirty cells per step, lanes 0 and 31 holding the neighbours
//    either side);
//  * along the x-row's slots, the running maximum of x from the first slot
//    and the running minimum from the last, kept at the last and the first
//    slot of each quad (slot 4g + 3 and 4g). A quad that straddles two x-rows
//    takes each value from the x-row that owns that slot; phase 1 reads a
//    quad's value only when that slot lies in the row it walks.
// fminf / fmaxf skip NaN coordinates, whose candidates every test rejects.
constexpr int kRowBoundsBlock = 256;

__global__ void __launch_bounds__(kRowBoundsBlock) k_row_bounds(DeviceState d, const float4 *__restrict__ pred)
{
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= d.xrows) return;  // whole warps
  int sg = 0;
  if (d.nseg > 1) {  // the last segment whose first x-row is <= w
    int lo = 0, hi = d.nseg - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (d.segs[mid].r_begin <= w) lo = mid; else hi = mid - 1;
    }
    sg = lo;
  }
  const SegParams &s = d.segs[sg];
  const int row = s.c_begin + (w - s.r_begin) * s.nx;
  const uint32_t *__restrict__ off = d.offsets;
  const unsigned full = 0xffffffffu;
  const float inf = __int_as_float(0x7f800000);
#pragma unroll 1
  for (int c0 = 0; c0 < s.nx; c0 += 30) {
    const int x = c0 - 1 + lane;
    float ylo = inf, yhi = -inf, zlo = inf, zhi = -inf;
    if (x >= 0 && x < s.nx) {
      const uint32_t a = __ldg(&off[row + x]), b = __ldg(&off[row + x + 1]);
      // the cell's particles eight at a time, their loads issued together
      // (past the cell's end a NaN, which fminf / fmaxf skip)
      const float nan = __int_as_float(0x7fc00000);
#pragma unroll 1
      for (uint32_t k = a; k < b; k += 8u) {
        float qy[8], qz[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          qy[u] = qz[u] = nan;
          if (k + u < b) {
            const float4 q = __ldg(&pred[k + u]);
            qy[u] = q.y;
            qz[u] = q.z;
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          ylo = fminf(ylo, qy[u]);
          yhi = fmaxf(yhi, qy[u]);
          zlo = fminf(zlo, qz[u]);
          zhi = fmaxf(zhi, qz[u]);
        }
      }
    }
    const float ylo_l = __shfl_up_sync(full, ylo, 1), ylo_r = __shfl_down_sync(full, ylo, 1);
    const float yhi_l = __shfl_up_sync(full, yhi, 1), yhi_r = __shfl_down_sync(full, yhi, 1);
    const float zlo_l = __shfl_up_sync(full, zlo, 1), zlo_r = __shfl_down_sync(full, zlo, 1);
    const float zhi_l = __shfl_up_sync(full, zhi, 1), zhi_r = __shfl_down_sync(full, zhi, 1);
    if (lane >= 1 && lane <= 30 && x < s.nx)
      d.row_yz[row + x] = make_float4(fminf(ylo, fminf(ylo_l, ylo_r)), fmaxf(yhi, fmaxf(yhi_l, yhi_r)),
                                      fminf(zlo, fminf(zlo_l, zlo_r)), fmaxf(zhi, fmaxf(zhi_l, zhi_r)));
  }
  const uint32_t A = __ldg(&off[row]), B = __ldg(&off[row + s.nx]);
  // running maximum from the first slot, eight 32-slot chunks per step (their
  // loads issued together)
  float carry = -inf;
#pragma unroll 1
  for (uint32_t b0 = A; b0 < B; b0 += 256u) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint32_t k = b0 + 32u * (uint32_t)u + (uint32_t)lane;
      v[u] = k < B ? __ldg(&pred[k]).x : -inf;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint32_t k = b0 + 32u * (uint32_t)u + (uint32_t)lane;
      float x = v[u];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(full, x, o);
        if (lane >= o) x = fmaxf(x, t);
      }
      x = fmaxf(x, carry);
      carry = __shfl_sync(full, x, 31);
      if (k < B && (k & 3u) == 3u) d.quad_bounds[k >> 2].x = x;
    }
  }
  // running minimum from the last slot
  carry = inf;
#pragma unroll 1
  for (uint32_t t0 = 0; t0 < B - A; t0 += 256u) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint32_t t = t0 + 32u * (uint32_t)u + (uint32_t)lane;  // slots from the x-row's last
      v[u] = t < B - A ? __ldg(&pred[B - 1u - t]).x : inf;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint32_t t = t0 + 32u * (uint32_t)u + (uint32_t)lane;
      const uint32_t k = B - 1u - t;
      float x = v[u];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float w = __shfl_up_sync(full, x, o);
        if (lane >= o) x = fminf(x, w);
      }
      x = fminf(x, carry);
      carry = __shfl_sync(full, x, 31);
      if (t < B - A && (k & 3u) == 0u) d.quad_bounds[k >> 2].y = x;
    }
  }
}

void launch_row_bounds(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  if (d.n <= 0 || d.xrows <= 0) return;
  const int warps = kRowBoundsBlock / 32;
  k_row_bounds<<<grid_for(d.xrows, warps), kRowBoundsBlock, 0, st>>>(d, pred);
}

// sph_xsph.glsl:35-81: c * sum (m / rho_j) (v_j - v_i) W(r), neighbour
// velocities from velj(k, pred_k). QUADS: d.quads holds pred (the fused
// substep), so phase 1 reads the quads. NORMALS (slots whose segment has
// sigma > 0): the same walk also evaluates sph_normal.glsl:24-81 for these
// positions, densities and grid - exactly the inputs the next substep's
// normal pass reads, since nothing between this pass and that one changes
// them - and leaves the result in *normal_out.
// The fused pass (QUADS) takes each neighbour's velocity and density from
// d.xv, left by the last delta_apply.
template <bool EXACT, bool QUADS, bool NORMALS, bool TRIMMED = false, class VelJ>
__device__ __forceinline__ float3 xsph_sum_f(const SegParams &s, const DeviceState &d, const float4 *__restrict__ pred,
                                             int i, float4 q, float3 vi, VelJ &&velj, float4 *normal_out = nullptr)
{
  const int3 base = cell_coord(s, q.x, q.y, q.z);
  const float h2 = s.h2, mass = s.mass, poly6 = s.poly6;
  const bool normals = NORMALS && s.sigma > 0.0f;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f, lap = 0.0f;
  auto body = [&](int k, bool within) {
    if (k == i) return;
    const float4 pj = __ldg(&pred[k]);
    const float dx = q.x - pj.x, dy = q.y - pj.y, dz = q.z - pj.z;
    const float r2 = pair_r2<EXACT>(dx, dy, dz);
    if (!within && r2 >= h2) return;
    float rho_j;
    float3 vj;
    if (QUADS) {
      const float4 xj = __ldg(&d.xv[k]);
      rho_j = xj.w;
      vj = make_float3(xj.x, xj.y, xj.z);
    } else {
      rho_j = fmaxf(__ldg(&d.lam[k].x), 1e-6f);
      vj = velj(k, pj);
    }
    if (EXACT) {
      const float w = mass / rho_j;
      const float wk = w_poly6(r2, h2, poly6);
      ax += (w * (vj.x - vi.x)) * wk;
      ay += (w * (vj.y - vi.y)) * wk;
      az += (w * (vj.z - vi.z)) * wk;
    } else {
      const float t = __fsub_rn(h2, r2);
      const float wk = __fmul_rn(__fdividef(s.mass_poly6, rho_j), __fmul_rn(__fmul_rn(t, t), t));
      ax = __fmaf_rn(wk, __fsub_rn(vj.x, vi.x), ax);
      ay = __fmaf_rn(wk, __fsub_rn(vj.y, vi.y), ay);
      az = __fmaf_rn(wk, __fsub_rn(vj.z, vi.z), az);
    }
    if (normals) normal_terms<EXACT>(s, rho_j, r2, dx, dy, dz, nx, ny, nz, lap);  // sph_normal.glsl's body
  };
  if (QUADS)
    for_each_within<EXACT, TRIMMED>(s, d.offsets, pred, d.quads, RowTrim{d.quad_bounds, d.row_yz}, q, h2, base, body);
  else
    for_each_within<EXACT>(s, d.offsets, pred, q, h2, base, body);
  if (normals) {
    const float mag = sqrtf(nx * nx + ny * ny + nz * nz);
    const float curv = (mag > 1e-4f) ? -lap / mag : 0.0f;
    *normal_out = make_float4(nx, ny, nz, curv);
  }
  const float c = s.visc;
  return make_float3(c * ax, c * ay, c * az);
}

// sph_velocity.glsl + sph_xsph.glsl + sph_finalize.glsl.
// NORMALS: also the next substep's normals, into d.normal_alt (the slot order
// of this grid, which the next substep's permute maps to its own). Bounded to
// five 256-thread blocks per SM (48 registers): with both bodies it spills at
// 40 (1.68 -> 1.63 ms per launch on the 4M-particle workload).
template <bool EXACT, bool NORMALS, int SEG, bool TRIMMED>
__global__ void __launch_bounds__(256, 5) k_xsph_finalize_f(DeviceState d, const float4 *__restrict__ pred,
                                                         float4 *__restrict__ pos_out, int keep_delta)
{
  FLOWX_SLOT_PROLOGUE_SEG
  const float4 q = pred[i];
  const float4 xi = d.xv[i];
  const float3 vi = make_float3(xi.x, xi.y, xi.z);
  const float3 dv = xsph_sum_f<EXACT, true, NORMALS, TRIMMED>(
      s, d, pred, i, q, vi, [](int, const float4 &) { return make_float3(0.f, 0.f, 0.f); }, d.normal_alt + i);
  float3 v = make_float3(vi.x + dv.x, vi.y + dv.y, vi.z + dv.z);
  float3 p = make_float3(q.x, q.y, q.z);
  finalize_particle(s, d.collider, p, v);
  pos_out[i] = make_float4(p.x, p.y, p.z, 1.0f);
  d.vel[i] = make_float4(v.x, v.y, v.z, 0.0f);
  if (keep_delta) d.delta[i] = make_float4(dv.x, dv.y, dv.z, 0.0f);
}

// sph_normal.glsl:24-81 (over the previous substep's grid, as the reference);
// the fused substep runs it only when the previous substep's XSPH pass did
// not already evaluate it (the first substep, or state changed in between).
template <bool EXACT, int SEG>
__global__ void __launch_bounds__(512, 3) k_normal_f(DeviceState d, const float4 *__restrict__ pred,
                                                  float4 *__restrict__ out)
{
  FLOWX_SLOT_PROLOGUE_SEG
  const float4 pi = pred[i];
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  const float h2 = s.h2;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f, lap = 0.0f;
  auto body = [&](int k, bool within) {
    if (k == i) return;
    const float4 pj = __ldg(&pred[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = pair_r2<EXACT>(dx, dy, dz);
    if (!within && r2 >= h2) return;
    normal_terms<EXACT>(s, fmaxf(__ldg(&d.lam[k].x), 1e-6f), r2, dx, dy, dz, nx, ny, nz, lap);
  };
  for_each_within<EXACT>(s, d.offsets, pred, pi, h2, base, body);
  const float mag = sqrtf(nx * nx + ny * ny + nz * nz);
  const float curv = (mag > 1e-4f) ? -lap / mag : 0.0f;
  out[i] = make_float4(nx, ny, nz, curv);
}

// f(std::bool_constant<TRIMMED>): the trimmed walk when the context's cells
// are coarser than the reach (d.trim), the plain row masks otherwise.
template <class F>
static void with_trimmed_walk(const DeviceState &d, F &&f)
{
  if (d.trim)
    f(std::true_type{});
  else
    f(std::false_type{});
}

void launch_lambda_f(const DeviceState &d, const float4 *pred, bool exact, cudaStream_t st)
{
  if (d.warp_passes) return launch_lambda_w(d, pred, exact, st);
  if (d.n <= 0) return;
  with_seg_source(d, [&](auto tag) {
    with_trimmed_walk(d, [&](auto wtag) {
      constexpr int SEG = decltype(tag)::value;
      constexpr bool TRIMMED = decltype(wtag)::value;
      const void *fn = exact ? (const void *)k_lambda_f<true, SEG, TRIMMED> : (const void *)k_lambda_f<false, SEG, TRIMMED>;
      const int b = FLOWX_BLOCK(d, K_LAMBDA, 128, fn);
      const unsigned g = grid_for(d.n, b);
      const size_t sh = TRIMMED ? trimmed_walk_bytes(b) : row_mask_bytes(b);
      if (exact) k_lambda_f<true, SEG, TRIMMED><<<g, b, sh, st>>>(d, pred);
      else k_lambda_f<false, SEG, TRIMMED><<<g, b, sh, st>>>(d, pred);
    });
  });
}
void launch_delta_apply_f(const DeviceState &d, const float4 *pred_in, float4 *pred_out, bool exact, bool last,
                          cudaStream_t st)
{
  if (d.warp_passes) return launch_delta_apply_w(d, pred_in, pred_out, exact, last, st);
  if (d.n <= 0) return;
  const int l = last ? 1 : 0;
  with_seg_source(d, [&](auto tag) {
    with_trimmed_walk(d, [&](auto wtag) {
      constexpr int SEG = decltype(tag)::value;
      constexpr bool TRIMMED = decltype(wtag)::value;
      const void *fn =
          exact ? (const void *)k_delta_apply_f<true, SEG, TRIMMED> : (const void *)k_delta_apply_f<false, SEG, TRIMMED>;
      const int b = FLOWX_BLOCK(d, K_DELTA_APPLY, 128, fn);
      const unsigned g = grid_for(d.n, b);
      if (exact) k_delta_apply_f<true, SEG, TRIMMED><<<g, b, row_mask_bytes(b), st>>>(d, pred_in, pred_out, l);
      else k_delta_apply_f<false, SEG, TRIMMED><<<g, b, row_mask_bytes(b), st>>>(d, pred_in, pred_out, l);
    });
  });
}
void launch_xsph_inputs(const DeviceState &d, const float4 *pred, bool exact, cudaStream_t st)
{
  if (d.n <= 0) return;
  if (exact) k_xsph_inputs<true><<<grid_for(d.n, 256), 256, 0, st>>>(d, pred);
  else k_xsph_inputs<false><<<grid_for(d.n, 256), 256, 0, st>>>(d, pred);
}
template <bool EXACT, bool NORMALS>
static void xsph_finalize_launch(const DeviceState &d, const float4 *pred, float4 *pos_out, int keep_delta,
                                 cudaStream_t st)
{
  with_seg_source(d, [&](auto tag) {
    with_trimmed_walk(d, [&](auto wtag) {
      constexpr int SEG = decltype(tag)::value;
      constexpr bool TRIMMED = decltype(wtag)::value;
      const void *fn = (const void *)k_xsph_finalize_f<EXACT, NORMALS, SEG, TRIMMED>;
      const int b = FLOWX_BLOCK(d, K_XSPH_FINALIZE, 128, fn);
      const size_t sh = TRIMMED ? trimmed_walk_bytes(b) : row_mask_bytes(b);
      k_xsph_finalize_f<EXACT, NORMALS, SEG, TRIMMED><<<grid_for(d.n, b), b, sh, st>>>(d, pred, pos_out, keep_delta);
    });
  });
}
void launch_xsph_finalize_f(const DeviceState &d, const float4 *pred, float4 *pos_out, bool keep_delta, bool exact,
                            bool normals, cudaStream_t st)
{
  if (d.warp_passes) return launch_xsph_finalize_w(d, pred, pos_out, keep_delta, exact, normals, st);
  if (d.n <= 0) return;
  const int kd = keep_delta ? 1 : 0;
  if (exact && normals) xsph_finalize_launch<true, true>(d, pred, pos_out, kd, st);
  else if (exact) xsph_finalize_launch<true, false>(d, pred, pos_out, kd, st);
  else if (normals) xsph_finalize_launch<false, true>(d, pred, pos_out, kd, st);
  else xsph_finalize_launch<false, false>(d, pred, pos_out, kd, st);
}
void launch_normal_f(const DeviceState &d, const float4 *pred, float4 *out, bool exact, cudaStream_t st)
{
  if (d.warp_passes) return launch_normal_w(d, pred, out, exact, st);
  if (d.n <= 0) return;
  with_seg_source(d, [&](auto tag) {
    constexpr int SEG = decltype(tag)::value;
    const void *fn = exact ? (const void *)k_normal_f<true, SEG> : (const void *)k_normal_f<false, SEG>;
    const int b = FLOWX_BLOCK(d, K_NORMAL, 128, fn);
    const unsigned g = grid_for(d.n, b);
    if (exact) k_normal_f<true, SEG><<<g, b, row_mask_bytes(b), st>>>(d, pred, out);
    else k_normal_f<false, SEG><<<g, b, row_mask_bytes(b), st>>>(d, pred, out);
  });
}

cudaError_t const_segs_upload_pbf(int base, const SegParams *s, int n, cudaStream_t st)
{
  return cudaMemcpyToSymbolAsync(c_segs, s, sizeof(SegParams) * n, sizeof(SegParams) * base, cudaMemcpyHostToDevice,
                                 st);
}

// ---- single reference passes (per-pass API; always exact) ------------------
// sph_predict.glsl:23-57
__global__ void k_predict(DeviceState d, float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE
  const float4 n = s.sigma > 0.0f ? d.normal[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  float3 vo, q;
  predict_particle(s, d.pos[i], d.vel[i], n, vo, q);
  d.vel[i] = make_float4(vo.x, vo.y, vo.z, 0.0f);
  pred[i] = make_float4(q.x, q.y, q.z, 1.0f);
}
// sph_delta.glsl:19-85
__global__ void __launch_bounds__(512) k_delta(DeviceState d, const float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE
  const float3 a = delta_sum_f<true, false>(s, d, pred, i, pred[i]);
  const float rest = s.rest;
  d.delta[i] = make_float4(a.x / rest, a.y / rest, a.z / rest, 0.0f);
}
// sph_apply_delta.glsl:10-20
__global__ void k_apply(DeviceState d, float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE
  (void)s;
  const float4 p = pred[i], dl = d.delta[i];
  pred[i] = make_float4(p.x + dl.x, p.y + dl.y, p.z + dl.z, 1.0f);
}
// sph_velocity.glsl:12-24
__global__ void k_velocity(DeviceState d, const float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE
  const float3 v = slot_velocity(pred[i], d.pos[i], s.dtc);
  d.vel[i] = make_float4(v.x, v.y, v.z, 0.0f);
}
// sph_xsph.glsl:28-82
__global__ void __launch_bounds__(512) k_xsph(DeviceState d, const float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE
  const float4 vi4 = d.vel[i];
  const float4 *__restrict__ vel = d.vel;
  const float3 dv = xsph_sum_f<true, false, false>(s, d, pred, i, pred[i], make_float3(vi4.x, vi4.y, vi4.z),
                                                  [&](int k, const float4 &) {
                                                    const float4 v = __ldg(&vel[k]);
                                                    return make_float3(v.x, v.y, v.z);
                                                  });
  d.delta[i] = make_float4(dv.x, dv.y, dv.z, 0.0f);
}
// sph_finalize.glsl:15-96
__global__ void k_finalize(DeviceState d, const float4 *__restrict__ pred)
{
  FLOWX_SLOT_PROLOGUE
  const float4 v4 = d.vel[i], dl = d.delta[i], q = pred[i];
  float3 v = make_float3(v4.x + dl.x, v4.y + dl.y, v4.z + dl.z);
  float3 p = make_float3(q.x, q.y, q.z);
  finalize_particle(s, d.collider, p, v);
  d.pos[i] = make_float4(p.x, p.y, p.z, 1.0f);
  d.vel[i] = make_float4(v.x, v.y, v.z, 0.0f);
}

void launch_normal(const DeviceState &d, const float4 *pred, float4 *out, cudaStream_t st)
{
  launch_normal_f(d, pred, out, true, st);
}
void launch_fill_quads(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  if (d.n > 0) k_fill_quads<<<grid_for(d.n, 256), 256, 0, st>>>(d, pred);
}
void launch_lambda(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  launch_fill_quads(d, pred, st);
  if (d.trim) launch_row_bounds(d, pred, st);
  launch_lambda_f(d, pred, true, st);
}
void launch_predict(const DeviceState &d, float4 *pred, cudaStream_t st)
{
  if (d.n > 0) k_predict<<<grid_for(d.n, 256), 256, 0, st>>>(d, pred);
}
void launch_delta(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  const int b = FLOWX_BLOCK(d, K_DELTA, 128, k_delta);
  if (d.n > 0) k_delta<<<grid_for(d.n, b), b, row_mask_bytes(b), st>>>(d, pred);
}
void launch_apply(const DeviceState &d, float4 *pred, cudaStream_t st)
{
  if (d.n > 0) k_apply<<<grid_for(d.n, 256), 256, 0, st>>>(d, pred);
}
void launch_velocity(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  if (d.n > 0) k_velocity<<<grid_for(d.n, 256), 256, 0, st>>>(d, pred);
}
void launch_xsph(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  const int b = FLOWX_BLOCK(d, K_XSPH, 128, k_xsph);
  if (d.n > 0) k_xsph<<<grid_for(d.n, b), b, row_mask_bytes(b), st>>>(d, pred);
}
void launch_finalize(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  if (d.n > 0) k_finalize<<<grid_for(d.n, 256), 256, 0, st>>>(d, pred);
}

// ---- per-frame density splat (surface_splat.glsl:32-97) -------------------
// One thread per lattice sample of one segment's surface grid; gathers the
// particles of the 5x5x5 cells around the sample's (clamped) cell.
struct SplatParams {
  float slox, sloy, sloz, spacing;
  float kh2, kcoef, mass, rest;
  int snx, sny, snz;
  int seg;
};

// Per-cell bounding box of the current positions (slots of the cell; an
// empty cell gets an inverted box). Used by the splat to skip cells that
// cannot reach a sample.
__global__ void k_cell_bounds(const uint32_t *__restrict__ off, const float4 *__restrict__ pos, int cells,
                              float4 *__restrict__ lo, float4 *__restrict__ hi)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cells) return;
  const uint32_t a = __ldg(&off[c]), b = __ldg(&off[c + 1]);
  float4 mn = make_float4(INFINITY, INFINITY, INFINITY, 0.0f), mx = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
  for (uint32_t k = a; k < b; ++k) {
    const float4 q = __ldg(&pos[k]);
    mn.x = fminf(mn.x, q.x);
    mn.y = fminf(mn.y, q.y);
    mn.z = fminf(mn.z, q.z);
    mx.x = fmaxf(mx.x, q.x);
    mx.y = fmaxf(mx.y, q.y);
    mx.z = fmaxf(mx.z, q.z);
  }
  lo[c] = mn;
  hi[c] = mx;
}

// One sample's offset to the nearest point of a box along one axis, with the
// sign the particle offsets (sample - particle) have there, 0 inside.
__device__ __forceinline__ float box_offset(float p, float lo, float hi)
{
  return p < lo ? p - lo : (p > hi ? p - hi : 0.0f);
}

// surface_splat.glsl:32-97: density / rest at every sample of the splat grid,
// from the particles of the 5x5x5 cells around the sample's cell in the
// reference's order (cells dz, dy, dx, slots ascending, MAX_CELL_SCAN per
// cell). A cell whose bounding box is at least the kernel radius away is
// skipped: every particle in it has r^2 >= the box's r^2 (subtraction,
// squaring and the sum round monotonically, and the box term uses the same
// expression), so each would add exactly mass * 0.
__global__ void __launch_bounds__(512) k_splat(DeviceState d, SplatParams sp, long long samples,
                                               float *__restrict__ out)
{
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= samples) return;
  const SegParams &s = d.segs[sp.seg];
  const int gx = (int)(t % sp.snx);
  const int gy = (int)((t / sp.snx) % sp.sny);
  const int gz = (int)(t / ((long long)sp.snx * sp.sny));
  const float px = sp.slox + (float)gx * sp.spacing;
  const float py = sp.sloy + (float)gy * sp.spacing;
  const float pz = sp.sloz + (float)gz * sp.spacing;
  const float h2 = sp.kh2, coef = sp.kcoef, mass = sp.mass;
  const float4 *__restrict__ pos = d.pos;
  float density = 0.0f;
  const int3 base = cell_coord(s, px, py, pz);
  constexpr int R = kSurfaceCellRadius;
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
#pragma unroll 1
      for (int x = x0; x <= x1; ++x) {
        const uint32_t cs = __ldg(&d.offsets[row + x]);
        uint32_t ce = __ldg(&d.offsets[row + x + 1]);
        if (ce == cs) continue;
        const float4 lo = __ldg(&d.cell_lo[row + x]), hi = __ldg(&d.cell_hi[row + x]);
        const float bx = box_offset(px, lo.x, hi.x), by = box_offset(py, lo.y, hi.y), bz = box_offset(pz, lo.z, hi.z);
        if (bx * bx + by * by + bz * bz >= h2) continue;
        if (ce - cs > (uint32_t)kMaxCellScan) ce = cs + kMaxCellScan;
#pragma unroll 1
        for (uint32_t k = cs; k < ce; ++k) {
          const float4 pj = __ldg(&pos[k]);
          const float dx = px - pj.x, dy2 = py - pj.y, dz2 = pz - pj.z;
          density += mass * w_poly6(dx * dx + dy2 * dy2 + dz2 * dz2, h2, coef);
        }
      }
    }
  }
  float value = density / fmaxf(sp.rest, 1e-6f);
  if (s.voxel > 0.0f) {
    const int3 c = collider_coord(s, px, py, pz);
    if (collider_occupied(s, d.collider, c.x, c.y, c.z)) value = 0.0f;
  }
  out[t] = value;
}

void launch_splat_segment(const DeviceState &d, int seg, int cell_begin, int cell_count, const float *surface_lo,
                          float spacing, float kernel_radius, float mass, float rest, const int *dims, float *out,
                          cudaStream_t st)
{
  SplatParams sp;
  sp.slox = surface_lo[0];
  sp.sloy = surface_lo[1];
  sp.sloz = surface_lo[2];
  sp.spacing = spacing;
  sp.kh2 = kernel_radius * kernel_radius;
  // sph_common.glsl:68-71 with the surface kernel radius (surface_splat.glsl:49-53)
  sp.kcoef = 315.0f / (64.0f * 3.14159265358979323846f * powf(kernel_radius, 9.0f));
  sp.mass = mass;
  sp.rest = rest;
  sp.snx = dims[0];
  sp.sny = dims[1];
  sp.snz = dims[2];
  sp.seg = seg;
  const long long samples = (long long)dims[0] * dims[1] * dims[2];
  if (cell_count > 0)
    k_cell_bounds<<<grid_for(cell_count, 256), 256, 0, st>>>(d.offsets + cell_begin, d.pos, cell_count,
                                                              d.cell_lo + cell_begin, d.cell_hi + cell_begin);
  const int b = FLOWX_BLOCK(d, K_SPLAT, 128, k_splat);
  if (samples > 0) k_splat<<<grid_for(samples, b), b, 0, st>>>(d, sp, samples, out);
}

// ---- analytic collider voxeliser --------------------------------------------
// Centre-inside occupancy of spheres, boxes and vertical cylinders, in double
// precision, on the reference's collider-grid layout (origin at the domain's
// low corner, x fastest: collision/__init__.py:245-254, :276-290).
struct DevPrimitive {
  int kind;  // 0 sphere, 1 box, 2 vertical cylinder (same layout as flowx_primitive)
  int pad;
  double a[3], b[3], r;
};

__global__ void k_voxelize(uint8_t *__restrict__ grid, int nx, int ny, int nz, double ox, double oy, double oz,
                           double voxel, const DevPrimitive *__restrict__ prims, int nprims)
{
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)nx * ny * nz;
  if (t >= total) return;
  const int x = (int)(t % nx), y = (int)((t / nx) % ny), z = (int)(t / ((long long)nx * ny));
  const double cx = ox + ((double)x + 0.5) * voxel;
  const double cy = oy + ((double)y + 0.5) * voxel;
  const double cz = oz + ((double)z + 0.5) * voxel;
  uint8_t occ = 0;
  for (int j = 0; j < nprims; ++j) {
    const DevPrimitive p = prims[j];
    if (p.kind == 0) {
      const double dx = cx - p.a[0], dy = cy - p.a[1], dz = cz - p.a[2];
      occ |= (dx * dx + dy * dy + dz * dz <= p.r * p.r) ? 1 : 0;
    } else if (p.kind == 1) {
      occ |= (cx >= p.a[0] && cx <= p.b[0] && cy >= p.a[1] && cy <= p.b[1] && cz >= p.a[2] && cz <= p.b[2]) ? 1
                                                                                                           : 0;
    } else if (p.kind == 2) {
      const double dx = cx - p.a[0], dy = cy - p.a[1];
      occ |= (dx * dx + dy * dy <= p.r * p.r && cz >= p.a[2] && cz <= p.b[2]) ? 1 : 0;
    }
  }
  grid[t] = occ;
}

void launch_voxelize(uint8_t *grid, int nx, int ny, int nz, float ox, float oy, float oz, float voxel,
                     const void *prims, int nprims, cudaStream_t st)
{
  const long long total = (long long)nx * ny * nz;
  if (total > 0)
    k_voxelize<<<grid_for(total, 256), 256, 0, st>>>(grid, nx, ny, nz, ox, oy, oz, voxel,
                                                     (const DevPrimitive *)prims, nprims);
}

}  // namespace flowx
