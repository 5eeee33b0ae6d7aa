// Buffers at the C ABI: device set-up, uploads and downloads in the
// reference's layouts, the collider grid, the splat, and per-kernel profiling.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "runtime.h"

namespace flowx {

static inline unsigned grid_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

__global__ void k_lam_from_f4(const uint32_t *__restrict__ ids, const float4 *__restrict__ by_id,
                              float2 *__restrict__ lam, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    const float4 v = by_id[ids[k]];
    lam[k] = make_float2(v.x, v.y);
  }
}
__global__ void k_lam_to_f4(const uint32_t *__restrict__ ids, const float2 *__restrict__ lam,
                            float4 *__restrict__ by_id, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    const float2 v = lam[k];
    by_id[ids[k]] = make_float4(v.x, v.y, 0.0f, 0.0f);
  }
}
__global__ void k_reorder_f2(const uint32_t *__restrict__ src_slot, const float2 *__restrict__ src,
                             float2 *__restrict__ dst, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = src[src_slot[k]];
}

int Ctx::init_device()
{
  int rc = cuda(cudaSetDevice(device), "cudaSetDevice");
  if (rc) return rc;
  rc = cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream create");
  if (rc) return rc;
  int sms = 0;
  rc = cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device attribute");
  if (rc) return rc;
  rc = allocate();
  d.sm_count = sms;
  return rc;
}

// Cell offsets for keys that were uploaded (rather than built): counted on
// the host from the uploaded key column once the cell count is known.
int Ctx::ensure_offsets()
{
  if (!offsets_dirty) return FLOWX_OK;
  const int cells = d.cells;
  std::vector<uint32_t> off((size_t)cells + 1, 0);
  for (int k = 0; k < total_particles; ++k) {
    if (h_keys[k] >= (uint32_t)cells)
      return fail(FLOWX_ERR_ARG, "uploaded keys hold a cell index >= the push block's cell_count");
    off[h_keys[k] + 1] += 1;
  }
  for (int c = 0; c < cells; ++c) off[c + 1] += off[c];
  int rc = cuda(cudaMemcpyAsync(d.offsets, off.data(), off.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                stream),
                "offsets upload");
  if (rc) return rc;
  rc = cuda(cudaStreamSynchronize(stream), "offsets upload");
  if (rc) return rc;
  offsets_dirty = false;
  have_grid = true;
  return FLOWX_OK;
}

// Move every per-particle array so that new slot k holds old slot src_slot[k].
int Ctx::reorder_state(const std::vector<uint32_t> &src_slot)
{
  next_normals_valid = false;
  const int n = total_particles;
  if (n == 0) return FLOWX_OK;
  int rc = cuda(cudaMemcpyAsync(d_src_slot, src_slot.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, stream),
                "reorder upload");
  if (rc) return rc;
  float4 *arrays[] = {d.pos, d.vel, d.pred_a, d.pred_b, d.normal, d.delta};
  for (float4 *a : arrays) {
    launch_reorder(d_src_slot, a, d.stage, n, stream);
    rc = cuda(cudaMemcpyAsync(a, d.stage, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream), "reorder copy");
    if (rc) return rc;
  }
  k_reorder_f2<<<grid_for(n, 256), 256, 0, stream>>>(d_src_slot, d.lam, d.lam_alt, n);
  g_launches += 7;
  rc = cuda(cudaMemcpyAsync(d.lam, d.lam_alt, n * sizeof(float2), cudaMemcpyDeviceToDevice, stream), "reorder copy");
  if (rc) return rc;
  return check_launch("reorder");
}

}  // namespace flowx

using namespace flowx;

static bool particle_f4_buffer(int b)
{
  return b == FLOWX_BUF_POSITIONS || b == FLOWX_BUF_VELOCITIES || b == FLOWX_BUF_PREDICTED ||
         b == FLOWX_BUF_DELTA || b == FLOWX_BUF_NORMAL;
}

static float4 *particle_ptr(Ctx *c, int b)
{
  switch (b) {
    case FLOWX_BUF_POSITIONS: return c->d.pos;
    case FLOWX_BUF_VELOCITIES: return c->d.vel;
    case FLOWX_BUF_PREDICTED: return c->pred_cur();
    case FLOWX_BUF_DELTA: return c->d.delta;
    case FLOWX_BUF_NORMAL: return c->d.normal;
    default: return nullptr;
  }
}

static int fetch_ids_keys(Ctx *c, std::vector<uint32_t> &ids, std::vector<uint32_t> &keys)
{
  const int n = c->total_particles;
  ids.resize(n);
  keys.resize(n);
  if (n == 0) return FLOWX_OK;
  int rc = c->cuda(cudaMemcpyAsync(ids.data(), c->d.ids, n * 4, cudaMemcpyDeviceToHost, c->stream), "ids download");
  if (rc) return rc;
  rc = c->cuda(cudaMemcpyAsync(keys.data(), c->d.keys, n * 4, cudaMemcpyDeviceToHost, c->stream), "keys download");
  if (rc) return rc;
  return c->cuda(cudaStreamSynchronize(c->stream), "download");
}

extern "C" {

int flowx_surface_field(flowx_ctx *ctx, const float **field, int64_t *samples)
{
  if (!ctx || !field || !samples) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  *field = c->d.surface;
  *samples = c->cap_samples;
  return FLOWX_OK;
}

int flowx_upload(flowx_ctx *ctx, int buffer, const void *host, size_t bytes)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  c->next_normals_valid = false;
  const int n = c->total_particles;
  if (!host && bytes) return c->fail(FLOWX_ERR_ARG, "host pointer is NULL");
  if (particle_f4_buffer(buffer) || buffer == FLOWX_BUF_LAMBDA) {
    if (bytes != (size_t)n * 16)
      return c->fail(FLOWX_ERR_ARG, "particle buffer upload must be particle_count * 16 bytes, got " +
                                        std::to_string(bytes));
    if (n == 0) return FLOWX_OK;
    int rc = c->cuda(cudaMemcpyAsync(c->d.stage, host, bytes, cudaMemcpyHostToDevice, c->stream), "upload");
    if (rc) return rc;
    if (buffer == FLOWX_BUF_NORMAL) {
      c->normal_in_order = true;
      c->normal_zero = false;
    }
    if (buffer == FLOWX_BUF_DELTA) c->delta_in_order = true;
    if (buffer == FLOWX_BUF_LAMBDA) {
      k_lam_from_f4<<<grid_for(n, 256), 256, 0, c->stream>>>(c->d.ids, c->d.stage, c->d.lam, n);
    } else {
      launch_gather_by_id(c->d.ids, c->d.stage, particle_ptr(c, buffer), n, c->stream);
    }
    g_launches += 1;
    rc = c->check_launch("upload");
    if (rc) return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "upload");
  }
  if (buffer == FLOWX_BUF_KEYS) {
    if (bytes % 16 != 0 || bytes / 16 < (size_t)n)
      return c->fail(FLOWX_ERR_ARG, "key upload must hold at least particle_count float4 entries");
    const float *f = static_cast<const float *>(host);
    std::vector<uint32_t> new_keys(n), new_ids(n);
    std::vector<char> seen(n, 0);
    for (int k = 0; k < n; ++k) {
      const float key = f[4 * k], id = f[4 * k + 1];
      if (!(key >= 0.0f) || !(id >= 0.0f) || key != std::floor(key) || id != std::floor(id) || id >= (float)n ||
          key >= (float)c->cap_cells)
        return c->fail(FLOWX_ERR_ARG, "key entry " + std::to_string(k) + " is not a valid (cell, particle id)");
      new_keys[k] = (uint32_t)key;
      new_ids[k] = (uint32_t)id;
      if (seen[new_ids[k]]) return c->fail(FLOWX_ERR_ARG, "particle id repeated in uploaded keys");
      seen[new_ids[k]] = 1;
      if (k > 0 && new_keys[k] < new_keys[k - 1])
        return c->fail(FLOWX_ERR_ARG, "uploaded keys are not sorted by cell");
    }
    std::vector<uint32_t> old_ids, old_keys;
    int rc = fetch_ids_keys(c, old_ids, old_keys);
    if (rc) return rc;
    std::vector<uint32_t> inv(n);
    for (int k = 0; k < n; ++k) inv[old_ids[k]] = (uint32_t)k;
    std::vector<uint32_t> src(n);
    for (int k = 0; k < n; ++k) src[k] = inv[new_ids[k]];
    rc = c->reorder_state(src);
    if (rc) return rc;
    if (n) {
      rc = c->cuda(cudaMemcpyAsync(c->d.ids, new_ids.data(), n * 4, cudaMemcpyHostToDevice, c->stream), "ids");
      if (rc) return rc;
      rc = c->cuda(cudaMemcpyAsync(c->d.keys, new_keys.data(), n * 4, cudaMemcpyHostToDevice, c->stream), "keys");
      if (rc) return rc;
    }
    c->h_keys = new_keys;
    c->keys_host_valid = true;
    c->offsets_dirty = true;
    c->have_grid = false;
    return c->cuda(cudaStreamSynchronize(c->stream), "key upload");
  }
  if (buffer == FLOWX_BUF_CELL_START || buffer == FLOWX_BUF_CELL_END) {
    // The ranges follow from the keys; an upload is checked against them.
    if (bytes % 4 != 0) return c->fail(FLOWX_ERR_ARG, "cell range upload must be whole floats");
    const int cells = (int)(bytes / 4);
    std::vector<uint32_t> keys;
    if (c->keys_host_valid) {
      keys = c->h_keys;
    } else {
      std::vector<uint32_t> ids;
      int rc = fetch_ids_keys(c, ids, keys);
      if (rc) return rc;
    }
    std::vector<float> want(cells, -1.0f);
    for (int k = 0; k < n; ++k) {
      const uint32_t key = keys[k];
      if (key >= (uint32_t)cells) return c->fail(FLOWX_ERR_ARG, "cell ranges shorter than the keys' cells");
      const bool first = k == 0 || keys[k - 1] != key;
      const bool last = k == n - 1 || keys[k + 1] != key;
      if (buffer == FLOWX_BUF_CELL_START && first) want[key] = (float)k;
      if (buffer == FLOWX_BUF_CELL_END && last) want[key] = (float)(k + 1);
    }
    if (std::memcmp(want.data(), host, bytes) != 0)
      return c->fail(FLOWX_ERR_ARG, "uploaded cell ranges do not match the keys");
    return FLOWX_OK;
  }
  return c->fail(FLOWX_ERR_ARG, "buffer " + std::to_string(buffer) + " cannot be uploaded");
}

int flowx_download(flowx_ctx *ctx, int buffer, void *host, size_t bytes)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  const int n = c->total_particles;
  if (!host && bytes) return c->fail(FLOWX_ERR_ARG, "host pointer is NULL");
  if (particle_f4_buffer(buffer) || buffer == FLOWX_BUF_LAMBDA) {
    if (bytes > (size_t)n * 16 || bytes % 16 != 0)
      return c->fail(FLOWX_ERR_ARG, "particle buffer download must be whole float4 entries, at most particle_count");
    if (bytes == 0) return FLOWX_OK;
    if ((buffer == FLOWX_BUF_NORMAL && !c->normal_in_order) || (buffer == FLOWX_BUF_DELTA && !c->delta_in_order))
      return c->fail(FLOWX_ERR_STATE, std::string(buffer == FLOWX_BUF_NORMAL ? "normal" : "delta") +
                                          " is scratch in the fused substep and no longer follows particle ids "
                                          "(create the context with FLOWX_FLAG_KEEP_DELTA to keep delta)");
    if (buffer == FLOWX_BUF_LAMBDA)
      k_lam_to_f4<<<grid_for(n, 256), 256, 0, c->stream>>>(c->d.ids, c->d.lam, c->d.stage, n);
    else
      launch_scatter_by_id(c->d.ids, particle_ptr(c, buffer), c->d.stage, n, c->stream);
    g_launches += 1;
    int rc = c->check_launch("download");
    if (rc) return rc;
    rc = c->cuda(cudaMemcpyAsync(host, c->d.stage, bytes, cudaMemcpyDeviceToHost, c->stream), "download");
    if (rc) return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "download");
  }
  if (buffer == FLOWX_BUF_KEYS) {
    if (bytes % 16 != 0) return c->fail(FLOWX_ERR_ARG, "key download must be whole float4 entries");
    int rc = c->ensure_offsets();
    if (rc) return rc;
    std::vector<uint32_t> ids, keys;
    rc = fetch_ids_keys(c, ids, keys);
    if (rc) return rc;
    const size_t m = bytes / 16;
    float *f = static_cast<float *>(host);
    const uint32_t cbegin = c->segs.empty() ? 0u : (uint32_t)c->segs[0].c_begin;
    for (size_t k = 0; k < m; ++k) {
      if (k < (size_t)n) {
        f[4 * k] = (float)(keys[k] - cbegin);
        f[4 * k + 1] = (float)ids[k];
      } else {
        f[4 * k] = (float)c->d.cells;  // padding slot (sph_grid_key.glsl:21-25)
        f[4 * k + 1] = (float)k;
      }
      f[4 * k + 2] = 0.0f;
      f[4 * k + 3] = 0.0f;
    }
    return FLOWX_OK;
  }
  if (buffer == FLOWX_BUF_CELL_START || buffer == FLOWX_BUF_CELL_END) {
    int rc = c->ensure_offsets();
    if (rc) return rc;
    if (bytes % 4 != 0 || bytes / 4 > (size_t)c->d.cells)
      return c->fail(FLOWX_ERR_ARG, "cell range download must be whole floats, at most cell_count");
    const size_t cells = bytes / 4;
    std::vector<uint32_t> off(cells + 1);
    if (cells) {
      rc = c->cuda(cudaMemcpyAsync(off.data(), c->d.offsets, (cells + 1) * 4, cudaMemcpyDeviceToHost, c->stream),
                   "offsets download");
      if (rc) return rc;
      rc = c->cuda(cudaStreamSynchronize(c->stream), "offsets download");
      if (rc) return rc;
    }
    float *f = static_cast<float *>(host);
    for (size_t q = 0; q < cells; ++q) {
      const bool empty = off[q + 1] == off[q];
      f[q] = empty ? -1.0f : (float)(buffer == FLOWX_BUF_CELL_START ? off[q] : off[q + 1]);
    }
    return FLOWX_OK;
  }
  if (buffer == FLOWX_BUF_SURFACE) {
    if (bytes % 4 != 0 || (long long)(bytes / 4) > c->cap_samples)
      return c->fail(FLOWX_ERR_ARG, "surface download larger than the splat grid capacity");
    if (!bytes) return FLOWX_OK;
    int rc = c->cuda(cudaMemcpyAsync(host, c->d.surface, bytes, cudaMemcpyDeviceToHost, c->stream), "download");
    if (rc) return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "download");
  }
  return c->fail(FLOWX_ERR_ARG, "unknown buffer id " + std::to_string(buffer));
}

int flowx_set_collider(flowx_ctx *ctx, const uint8_t *occupancy, const int32_t dims[3], float voxel_size)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  if (!occupancy || !(voxel_size > 0.0f)) {
    c->collider_installed = false;
    return FLOWX_OK;
  }
  if (!dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
    return c->fail(FLOWX_ERR_ARG, "collider dims must be positive");
  const long long voxels = (long long)dims[0] * dims[1] * dims[2];
  if (voxels > c->cap_voxels)
    return c->fail(FLOWX_ERR_CAPACITY, "collider grid larger than max_collider_voxels");
  int rc = c->cuda(cudaMemcpyAsync(c->d.collider, occupancy, (size_t)voxels, cudaMemcpyHostToDevice, c->stream),
                   "collider upload");
  if (rc) return rc;
  c->collider_installed = true;
  std::memcpy(c->collider_dims, dims, sizeof(c->collider_dims));
  return c->cuda(cudaStreamSynchronize(c->stream), "collider upload");
}

int flowx_voxelize(flowx_ctx *ctx, const flowx_primitive *prims, int count, const int32_t dims[3],
                   float voxel_size, const float origin[3])
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  if (count < 0 || (count > 0 && !prims) || !dims || !origin || !(voxel_size > 0.0f))
    return c->fail(FLOWX_ERR_ARG, "bad voxelize arguments");
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return c->fail(FLOWX_ERR_ARG, "collider dims must be positive");
  const long long voxels = (long long)dims[0] * dims[1] * dims[2];
  if (voxels > c->cap_voxels) return c->fail(FLOWX_ERR_CAPACITY, "collider grid larger than max_collider_voxels");
  if (count > c->prim_cap) {
    if (c->d_prims) cudaFree(c->d_prims);
    c->d_prims = nullptr;
    int rc = c->cuda(cudaMalloc(&c->d_prims, sizeof(flowx_primitive) * (size_t)count), "primitive buffer");
    if (rc) return rc;
    c->prim_cap = count;
  }
  if (count) {
    int rc = c->cuda(cudaMemcpyAsync(c->d_prims, prims, sizeof(flowx_primitive) * (size_t)count,
                                     cudaMemcpyHostToDevice, c->stream),
                     "primitive upload");
    if (rc) return rc;
  }
  launch_voxelize(c->d.collider, dims[0], dims[1], dims[2], origin[0], origin[1], origin[2], voxel_size, c->d_prims,
                  count, c->stream);
  g_launches += 1;
  c->collider_installed = true;
  std::memcpy(c->collider_dims, dims, sizeof(c->collider_dims));
  return c->check_launch("flowx_voxelize");
}

int flowx_splat(flowx_ctx *ctx, const flowx_push *push, float *host_out, size_t bytes)
{
  if (!ctx || !push) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  const int dims[3] = {push->i_sort[0], push->i_sort[1], push->i_sort[2]};
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return c->fail(FLOWX_ERR_ARG, "splat sample dims must be > 0");
  const long long samples = (long long)dims[0] * dims[1] * dims[2];
  if (samples > c->cap_samples) return c->fail(FLOWX_ERR_CAPACITY, "splat grid larger than max_surface_samples");
  if (host_out && bytes != (size_t)samples * 4)
    return c->fail(FLOWX_ERR_ARG, "splat output must be samples * 4 bytes");
  // The splat block shares the solver block's geometry rows (f_lo, i_grid,
  // i_collider); its repurposed rows are read here, not as solver values.
  int rc = c->set_push(push);
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  if (!c->have_grid) return c->fail(FLOWX_ERR_STATE, "splat before any grid build");
  launch_splat_segment(c->d, 0, c->segs[0].c_begin, c->segs[0].c_count, push->f_hi, bits_to_float(push->i_sort[3]),
                       push->f_sph[0], push->f_sph[1], push->f_sph[2], dims, c->d.surface, c->stream);
  g_launches += 2;
  rc = c->check_launch("flowx_splat");
  if (rc) return rc;
  if (host_out) {
    rc = c->cuda(cudaMemcpyAsync(host_out, c->d.surface, bytes, cudaMemcpyDeviceToHost, c->stream), "splat download");
    if (rc) return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "splat download");
  }
  return FLOWX_OK;
}

int flowx_profile_substeps(flowx_ctx *ctx, const flowx_push *push, int iterations, int substeps, float *ms,
                           int32_t *launches)
{
  if (!ctx || !ms || !launches || substeps < 1 || iterations < 0) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  int rc = c->set_push(push);
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  return c->profile_substeps(iterations, substeps, ms, launches);
}

}  // extern "C"

// Fused substeps issued launch by launch with CUDA events around every
// kernel; adds milliseconds and launch counts per kernel id.
int Ctx::profile_substeps(int iterations, int substeps, float *ms, int32_t *launches)
{
  Ctx *c = this;
  int rc = c->ensure_grid();
  if (rc) return rc;
  struct Rec {
    int kid, count;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  auto timed = [&](int kid, int count, auto fn) {
    Rec r{kid, count, nullptr, nullptr};
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, c->stream);
    fn();
    cudaEventRecord(r.b, c->stream);
    recs.push_back(r);
  };
  const DeviceState &d = c->d;
  const bool exact = (c->flags & FLOWX_FLAG_EXACT) != 0;
  const int end_idx = iterations % 2 == 0 ? 0 : 1;
  for (int s = 0; s < substeps; ++s) {
    float4 *pin = c->pred_cur();
    const bool sigma = c->segs_need_normal();
    if (sigma && !c->next_normals_valid)
      timed(K_NORMAL, 1, [&] { launch_normal_f(d, pin, d.normal_alt, exact, c->stream); });
    timed(K_PREDICT_KEY, 1, [&] { launch_predict_key(d, d.normal_alt, c->stream); });
    timed(K_SCAN_REDUCE, 3, [&] { launch_scan(d, c->stream); });
    if (c->flags & FLOWX_FLAG_REFERENCE_ORDER) {
      int launched = 0;
      timed(K_BITONIC, 0, [&] { launched = launch_reference_order(d, c->stream); });
      launches[K_BITONIC] += launched;
      g_launches += launched;
    } else {
      timed(K_SCATTER, 1, [&] { launch_scatter(d, c->stream, d.x_order != 0); });
      timed(K_CELL_SORT_SMALL, 2, [&] { launch_cell_sort(d, c->stream); });
    }
    timed(K_PERMUTE_STEP, 1, [&] { launch_permute_step(d, d.pred_a, d.normal_alt, c->stream); });
    float4 *q_in = d.pred_a, *q_out = d.pred_b;
    for (int it = 0; it < iterations; ++it) {
      if (d.trim) timed(K_ROW_BOUNDS, 1, [&] { launch_row_bounds(d, q_in, c->stream); });
      timed(K_LAMBDA, 1, [&] { launch_lambda_f(d, q_in, exact, c->stream); });
      const bool last = it == iterations - 1;
      timed(K_DELTA_APPLY, 1, [&] { launch_delta_apply_f(d, q_in, q_out, exact, last, c->stream); });
      std::swap(q_in, q_out);
      if (d.trim) std::swap(c->d.quads, c->d.quads_alt);  // d aliases c->d
    }
    if (iterations == 0) launch_xsph_inputs(d, q_in, exact, c->stream);
    if (d.trim) timed(K_ROW_BOUNDS, 1, [&] { launch_row_bounds(d, q_in, c->stream); });
    timed(K_XSPH_FINALIZE, 1, [&] {
      launch_xsph_finalize_f(d, q_in, d.pos, (c->flags & FLOWX_FLAG_KEEP_DELTA) != 0, exact, sigma,
                             c->stream);
    });
    c->pred_idx = end_idx;
    c->after_fused_substep();
  }
  rc = c->cuda(cudaStreamSynchronize(c->stream), "profile");
  for (auto &r : recs) {
    float t = 0.0f;
    cudaEventElapsedTime(&t, r.a, r.b);
    ms[r.kid] += t;
    launches[r.kid] += r.count;
    g_launches += r.count;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  c->keys_host_valid = false;
  if (rc) return rc;
  return c->check_launch("flowx_profile_substeps");
}
