// Warp-per-particle neighbour passes, for scenes too small to fill the GPU
// with one thread per particle.
//
// With one thread per particle, a 3,200-particle scene runs 25 blocks of 128
// threads on 152 SMs, and each thread walks its ~250 candidates one after
// another: the passes wait on dependent loads, not on issue. Here a warp takes
// one particle. For each of the nine (dz, dy) stencil rows its lanes test 32
// consecutive candidate slots at once (one coalesced load per lane). The
// accepted candidates' terms are computed in parallel, then folded into the
// particle's sums lane by lane in slot order (a ballot, then one shuffle per
// value): the same operations in the same order as the thread-per-particle
// kernels of pbf.cu, so both give bit-identical results in both arithmetic
// modes. Rows whose run exceeds the reference's MAX_CELL_SCAN are walked cell
// by cell with the cap, as the reference does.
//
// The passes: normal (sph_normal.glsl), lambda (sph_lambda.glsl), delta_apply
// (sph_delta.glsl + sph_apply_delta.glsl) and xsph_finalize (sph_velocity +
// sph_xsph + sph_finalize, with the next substep's normal pass fused), each
// with the pbf.cu kernel's inputs and outputs.
#include "neighbour.cuh"

namespace flowx {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarpBlock = 128;  // four particles per block

inline unsigned warp_grid(int n) { return (unsigned)(((long long)n * 32 + kWarpBlock - 1) / kWarpBlock); }

template <class Test, class Add>
__device__ __forceinline__ void walk_run(uint32_t a, uint32_t b, int lane, Test &test, Add &add)
{
#pragma unroll 1
  for (uint32_t c0 = a; c0 < b; c0 += 32u) {
    const uint32_t k = c0 + (uint32_t)lane;
    const bool take = k < b && test((int)k);
    unsigned m = __ballot_sync(kFull, take);
#pragma unroll 1
    while (m) {
      const int l = __ffs(m) - 1;
      m &= m - 1u;
      add(l);
    }
  }
}

// Every candidate slot of the 27-cell stencil around `base`, in the
// reference's order (rows dz, dy; slots ascending; MAX_CELL_SCAN per cell).
// test(k): lane-local, true when slot k contributes, leaving the lane's term
// values; add(l): all lanes fold lane l's values into their (identical)
// sums, called once per contributing slot, in slot order.
template <class Test, class Add>
__device__ __forceinline__ void warp_walk(const SegParams &s, const uint32_t *__restrict__ off, int3 base,
                                          Test &&test, Add &&add)
{
  const int lane = threadIdx.x & 31;
  const int x0 = max(base.x - 1, 0), x1 = min(base.x + 1, s.nx - 1);
  uint32_t ra_l = 0, rb_l = 0;
  int row_l = 0;
  if (lane < kRows) {
    const int z = base.z + lane / 3 - 1, y = base.y + lane % 3 - 1;
    if (z >= 0 && z < s.nz && y >= 0 && y < s.ny) {
      row_l = s.c_begin + (z * s.ny + y) * s.nx;
      ra_l = __ldg(&off[row_l + x0]);
      rb_l = __ldg(&off[row_l + x1 + 1]);
    }
  }
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const uint32_t ra = __shfl_sync(kFull, ra_l, r), rb = __shfl_sync(kFull, rb_l, r);
    if (rb <= ra) continue;
    if (rb - ra <= (uint32_t)kMaxCellScan) {
      walk_run(ra, rb, lane, test, add);
    } else {
      const int row = __shfl_sync(kFull, row_l, r);
#pragma unroll 1
      for (int x = x0; x <= x1; ++x) {
        const uint32_t cs = __ldg(&off[row + x]);
        uint32_t ce = __ldg(&off[row + x + 1]);
        if (ce - cs > (uint32_t)kMaxCellScan) ce = cs + kMaxCellScan;
        walk_run(cs, ce, lane, test, add);
      }
    }
  }
}

__device__ __forceinline__ float shfl(float v, int l) { return __shfl_sync(kFull, v, l); }

#define FLOWX_WARP_PROLOGUE                                          \
  const int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); \
  if (i >= d.n) return;                                              \
  const int lane = threadIdx.x & 31;                                 \
  const SegParams &s = slot_params<SEG>(d, i);

// sph_lambda.glsl:17-77; LambdaAcc's operations (neighbour.cuh), folded per
// candidate: the density term for every candidate within h, the gradient
// terms for those with r^2 > 1e-12.
template <bool EXACT, int SEG>
__global__ void __launch_bounds__(kWarpBlock) k_lambda_w(DeviceState d, const float4 *__restrict__ pred)
{
  FLOWX_WARP_PROLOGUE
  const float4 pi = pred[i];
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  LambdaAcc<EXACT> acc;
  float ta = 0.f, tb = 0.f, tc = 0.f, td = 0.f, te = 0.f, tf = 0.f, tg = 0.f, th = 0.f;
  bool grad = false;
  auto test = [&](int k) -> bool {
    const float4 pj = __ldg(&pred[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = pair_r2<EXACT>(dx, dy, dz);
    if (r2 >= s.h2) return false;
    grad = r2 > 1e-12f;
    if (EXACT) {
      ta = s.mass * w_poly6(r2, s.h2, s.poly6);
      if (grad) {
        const float r = sqrtf(r2);
        const float sg = s.mass * w_spiky_grad(r, s.h, s.spiky);
        tb = sg * (dx / r);
        tc = sg * (dy / r);
        td = sg * (dz / r);
        te = tb * tb + tc * tc + td * td;
      }
    } else {
      const float t = __fsub_rn(s.h2, r2);
      ta = __fmul_rn(t, t);
      tb = t;
      if (grad) {
        const float rinv = rsqrtf(r2);
        const float hr = __fsub_rn(s.h, __fmul_rn(r2, rinv));
        const float g = __fmul_rn(__fmul_rn(s.mass_spiky, __fmul_rn(hr, hr)), rinv);
        tc = g;
        td = dx;
        te = dy;
        tf = dz;
        tg = __fmul_rn(g, g);
        th = r2;
      }
    }
    return true;
  };
  auto add = [&](int l) {
    const bool gl = __shfl_sync(kFull, grad ? 1 : 0, l) != 0;
    if (EXACT) {
      acc.density += shfl(ta, l);
      if (gl) {
        acc.gx += shfl(tb, l);
        acc.gy += shfl(tc, l);
        acc.gz += shfl(td, l);
        acc.gn2 += shfl(te, l);
      }
    } else {
      acc.density = __fmaf_rn(shfl(ta, l), shfl(tb, l), acc.density);
      if (gl) {
        const float g = shfl(tc, l);
        acc.gx = __fmaf_rn(g, shfl(td, l), acc.gx);
        acc.gy = __fmaf_rn(g, shfl(te, l), acc.gy);
        acc.gz = __fmaf_rn(g, shfl(tf, l), acc.gz);
        acc.gn2 = __fmaf_rn(shfl(tg, l), shfl(th, l), acc.gn2);
      }
    }
  };
  warp_walk(s, d.offsets, base, test, add);
  if (lane == 0) {
    const float2 lm = acc.finish(s);
    d.lam[i] = lm;
    d.plam[i] = make_float4(pi.x, pi.y, pi.z, lm.y);
  }
}

// sph_delta.glsl:19-85 + sph_apply_delta.glsl; delta_pair's operations
// (neighbour.cuh), folded per candidate with 1e-12 < r^2 < h^2.
template <bool EXACT, int SEG>
__global__ void __launch_bounds__(kWarpBlock) k_delta_apply_w(DeviceState d, const float4 *__restrict__ pred_in,
                                                              float4 *__restrict__ pred_out, int last)
{
  FLOWX_WARP_PROLOGUE
  const float4 pi = pred_in[i];
  const float lambda_i = d.lam[i].y;
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  float ta = 0.f, tb = 0.f, tc = 0.f, td = 0.f;
  auto test = [&](int k) -> bool {
    const float4 pj = __ldg(&pred_in[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = pair_r2<EXACT>(dx, dy, dz);
    if (r2 >= s.h2 || r2 <= 1e-12f) return false;
    const float lambda_j = __ldg(&d.lam[k].y);
    if (EXACT) {
      const float r = sqrtf(r2);
      float s_corr = 0.0f;
      if (s.scorr_k > 0.0f && s.w_q > 1e-9f) {
        const float ratio = w_poly6(r2, s.h2, s.poly6) / s.w_q;
        const float rr = fmaxf(ratio, 0.0f);
        const float rr2 = rr * rr;
        s_corr = -s.scorr_k * (rr2 * rr2);
      }
      const float sc = (lambda_i + lambda_j + s_corr) * w_spiky_grad(r, s.h, s.spiky);
      ta = sc * (dx / r);
      tb = sc * (dy / r);
      tc = sc * (dz / r);
    } else {
      const float rinv = rsqrtf(r2);
      const float hr = __fsub_rn(s.h, __fmul_rn(r2, rinv));
      float lam = __fadd_rn(lambda_i, lambda_j);
      if (s.scorr_k > 0.0f && s.w_q > 1e-9f) {
        const float t = __fsub_rn(s.h2, r2);
        const float ratio = __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), s.poly6_over_wq);
        const float rr2 = __fmul_rn(ratio, ratio);
        lam = __fmaf_rn(-s.scorr_k, __fmul_rn(rr2, rr2), lam);
      }
      ta = __fmul_rn(__fmul_rn(lam, __fmul_rn(s.spiky, __fmul_rn(hr, hr))), rinv);
      tb = dx;
      tc = dy;
      td = dz;
    }
    return true;
  };
  auto add = [&](int l) {
    if (EXACT) {
      ax += shfl(ta, l);
      ay += shfl(tb, l);
      az += shfl(tc, l);
    } else {
      const float sc = shfl(ta, l);
      ax = __fmaf_rn(sc, shfl(tb, l), ax);
      ay = __fmaf_rn(sc, shfl(tc, l), ay);
      az = __fmaf_rn(sc, shfl(td, l), az);
    }
  };
  warp_walk(s, d.offsets, base, test, add);
  if (lane == 0) {
    const float rest = s.rest;
    const float4 q = make_float4(pi.x + ax / rest, pi.y + ay / rest, pi.z + az / rest, 1.0f);
    pred_out[i] = q;
    store_quad(d.quads, i, q.x, q.y, q.z);
    if (last) d.xv[i] = xsph_input<EXACT>(s, d, i, q);
  }
}

// The normal pass's per-neighbour terms (normal_terms, pbf.cu) as values a
// lane hands to the fold: EXACT the four summands; FAST the factors of its
// four fused multiply-adds (sg and the offset for n, the weight and h - r
// for the laplacian).
struct NormalTerm {
  float a, b, c, d, e, f;

  template <bool EXACT>
  __device__ __forceinline__ void make(const SegParams &s, float rho_j, float r2, float dx, float dy, float dz)
  {
    if (EXACT) {
      const float weight = s.mass / rho_j;
      const float t = s.h2 - r2;
      const float sg = s.poly6m6 * t * t;
      a = weight * (sg * dx);
      b = weight * (sg * dy);
      c = weight * (sg * dz);
      d = weight * w_visc_lap(sqrtf(r2), s.h, s.visclap);
    } else {
      const float weight = __fdividef(s.mass, rho_j);
      const float t = __fsub_rn(s.h2, r2);
      a = __fmul_rn(weight, __fmul_rn(s.poly6m6, __fmul_rn(t, t)));
      b = dx;
      c = dy;
      d = dz;
      const float r = r2 > 0.0f ? __fmul_rn(r2, rsqrtf(r2)) : 0.0f;
      e = __fmul_rn(weight, s.visclap);
      f = __fsub_rn(s.h, r);
    }
  }

  template <bool EXACT>
  __device__ __forceinline__ void fold(int l, float &nx, float &ny, float &nz, float &lap) const
  {
    if (EXACT) {
      nx += shfl(a, l);
      ny += shfl(b, l);
      nz += shfl(c, l);
      lap += shfl(d, l);
    } else {
      const float sg = shfl(a, l);
      nx = __fmaf_rn(sg, shfl(b, l), nx);
      ny = __fmaf_rn(sg, shfl(c, l), ny);
      nz = __fmaf_rn(sg, shfl(d, l), nz);
      lap = __fmaf_rn(shfl(e, l), shfl(f, l), lap);
    }
  }
};

// sph_velocity.glsl + sph_xsph.glsl + sph_finalize.glsl as k_xsph_finalize_f
// (pbf.cu), neighbour velocities and densities from d.xv; NORMALS: also the
// next substep's normal pass into d.normal_alt.
template <bool EXACT, bool NORMALS, int SEG>
__global__ void __launch_bounds__(kWarpBlock) k_xsph_finalize_w(DeviceState d, const float4 *__restrict__ pred,
                                                                float4 *__restrict__ pos_out, int keep_delta)
{
  FLOWX_WARP_PROLOGUE
  const float4 q = pred[i];
  const float4 xi = d.xv[i];
  const float3 vi = make_float3(xi.x, xi.y, xi.z);
  const int3 base = cell_coord(s, q.x, q.y, q.z);
  const bool normals = NORMALS && s.sigma > 0.0f;
  float ax = 0.0f, ay = 0.0f, az = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, lap = 0.0f;
  float ta = 0.f, tb = 0.f, tc = 0.f, td = 0.f;
  NormalTerm nt{};
  auto test = [&](int k) -> bool {
    if (k == i) return false;
    const float4 pj = __ldg(&pred[k]);
    const float dx = q.x - pj.x, dy = q.y - pj.y, dz = q.z - pj.z;
    const float r2 = pair_r2<EXACT>(dx, dy, dz);
    if (r2 >= s.h2) return false;
    const float4 xj = __ldg(&d.xv[k]);
    const float rho_j = xj.w;
    if (EXACT) {
      const float w = s.mass / rho_j;
      const float wk = w_poly6(r2, s.h2, s.poly6);
      ta = (w * (xj.x - vi.x)) * wk;
      tb = (w * (xj.y - vi.y)) * wk;
      tc = (w * (xj.z - vi.z)) * wk;
    } else {
      const float t = __fsub_rn(s.h2, r2);
      ta = __fmul_rn(__fdividef(s.mass_poly6, rho_j), __fmul_rn(__fmul_rn(t, t), t));
      tb = __fsub_rn(xj.x, vi.x);
      tc = __fsub_rn(xj.y, vi.y);
      td = __fsub_rn(xj.z, vi.z);
    }
    if (normals) nt.make<EXACT>(s, rho_j, r2, dx, dy, dz);
    return true;
  };
  auto add = [&](int l) {
    if (EXACT) {
      ax += shfl(ta, l);
      ay += shfl(tb, l);
      az += shfl(tc, l);
    } else {
      const float wk = shfl(ta, l);
      ax = __fmaf_rn(wk, shfl(tb, l), ax);
      ay = __fmaf_rn(wk, shfl(tc, l), ay);
      az = __fmaf_rn(wk, shfl(td, l), az);
    }
    if (normals) nt.fold<EXACT>(l, nx, ny, nz, lap);
  };
  warp_walk(s, d.offsets, base, test, add);
  if (lane != 0) return;
  if (normals) {
    const float mag = sqrtf(nx * nx + ny * ny + nz * nz);
    const float curv = (mag > 1e-4f) ? -lap / mag : 0.0f;
    d.normal_alt[i] = make_float4(nx, ny, nz, curv);
  }
  const float c = s.visc;
  const float3 dv = make_float3(c * ax, c * ay, c * az);
  float3 v = make_float3(vi.x + dv.x, vi.y + dv.y, vi.z + dv.z);
  float3 p = make_float3(q.x, q.y, q.z);
  finalize_particle(s, d.collider, p, v);
  pos_out[i] = make_float4(p.x, p.y, p.z, 1.0f);
  d.vel[i] = make_float4(v.x, v.y, v.z, 0.0f);
  if (keep_delta) d.delta[i] = make_float4(dv.x, dv.y, dv.z, 0.0f);
}

// sph_normal.glsl:24-81 as k_normal_f (pbf.cu).
template <bool EXACT, int SEG>
__global__ void __launch_bounds__(kWarpBlock) k_normal_w(DeviceState d, const float4 *__restrict__ pred,
                                                         float4 *__restrict__ out)
{
  FLOWX_WARP_PROLOGUE
  const float4 pi = pred[i];
  const int3 base = cell_coord(s, pi.x, pi.y, pi.z);
  float nx = 0.0f, ny = 0.0f, nz = 0.0f, lap = 0.0f;
  NormalTerm nt{};
  auto test = [&](int k) -> bool {
    if (k == i) return false;
    const float4 pj = __ldg(&pred[k]);
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = pair_r2<EXACT>(dx, dy, dz);
    if (r2 >= s.h2) return false;
    nt.make<EXACT>(s, fmaxf(__ldg(&d.lam[k].x), 1e-6f), r2, dx, dy, dz);
    return true;
  };
  auto add = [&](int l) { nt.fold<EXACT>(l, nx, ny, nz, lap); };
  warp_walk(s, d.offsets, base, test, add);
  if (lane == 0) {
    const float mag = sqrtf(nx * nx + ny * ny + nz * nz);
    const float curv = (mag > 1e-4f) ? -lap / mag : 0.0f;
    out[i] = make_float4(nx, ny, nz, curv);
  }
}

}  // namespace

void launch_lambda_w(const DeviceState &d, const float4 *pred, bool exact, cudaStream_t st)
{
  if (d.n <= 0) return;
  with_seg_source(d, [&](auto tag) {
    constexpr int SEG = decltype(tag)::value;
    if (exact) k_lambda_w<true, SEG><<<warp_grid(d.n), kWarpBlock, 0, st>>>(d, pred);
    else k_lambda_w<false, SEG><<<warp_grid(d.n), kWarpBlock, 0, st>>>(d, pred);
  });
}
void launch_delta_apply_w(const DeviceState &d, const float4 *pred_in, float4 *pred_out, bool exact, bool last,
                          cudaStream_t st)
{
  if (d.n <= 0) return;
  const int l = last ? 1 : 0;
  with_seg_source(d, [&](auto tag) {
    constexpr int SEG = decltype(tag)::value;
    if (exact) k_delta_apply_w<true, SEG><<<warp_grid(d.n), kWarpBlock, 0, st>>>(d, pred_in, pred_out, l);
    else k_delta_apply_w<false, SEG><<<warp_grid(d.n), kWarpBlock, 0, st>>>(d, pred_in, pred_out, l);
  });
}
template <bool EXACT, bool NORMALS>
static void xsph_finalize_w_launch(const DeviceState &d, const float4 *pred, float4 *pos_out, int kd, cudaStream_t st)
{
  with_seg_source(d, [&](auto tag) {
    constexpr int SEG = decltype(tag)::value;
    k_xsph_finalize_w<EXACT, NORMALS, SEG><<<warp_grid(d.n), kWarpBlock, 0, st>>>(d, pred, pos_out, kd);
  });
}
void launch_xsph_finalize_w(const DeviceState &d, const float4 *pred, float4 *pos_out, bool keep_delta, bool exact,
                            bool normals, cudaStream_t st)
{
  if (d.n <= 0) return;
  const int kd = keep_delta ? 1 : 0;
  if (exact && normals) xsph_finalize_w_launch<true, true>(d, pred, pos_out, kd, st);
  else if (exact) xsph_finalize_w_launch<true, false>(d, pred, pos_out, kd, st);
  else if (normals) xsph_finalize_w_launch<false, true>(d, pred, pos_out, kd, st);
  else xsph_finalize_w_launch<false, false>(d, pred, pos_out, kd, st);
}
void launch_normal_w(const DeviceState &d, const float4 *pred, float4 *out, bool exact, cudaStream_t st)
{
  if (d.n <= 0) return;
  with_seg_source(d, [&](auto tag) {
    constexpr int SEG = decltype(tag)::value;
    if (exact) k_normal_w<true, SEG><<<warp_grid(d.n), kWarpBlock, 0, st>>>(d, pred, out);
    else k_normal_w<false, SEG><<<warp_grid(d.n), kWarpBlock, 0, st>>>(d, pred, out);
  });
}

cudaError_t const_segs_upload_warp(int base, const SegParams *s, int n, cudaStream_t st)
{
  return cudaMemcpyToSymbolAsync(c_segs, s, sizeof(SegParams) * n, sizeof(SegParams) * base, cudaMemcpyHostToDevice,
                                 st);
}

}  // namespace flowx
