// Batched scenes and the block-size autotuner (C ABI in include/flowx.h).
//
// A batch is one context holding several independent scenes. Their particles
// (in scene order), cells and collider voxels are concatenated; each scene's
// push block becomes one entry of the device segment table. Sort keys carry
// the scene's cell offset, so the counting sort never mixes scenes and every
// kernel of the substep serves all scenes in one launch, looking up its
// scene's parameters per slot. No reference counterpart: the reference
// simulates one domain per Blender scene (README.md:141).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "runtime.h"

using namespace flowx;

namespace {

Ctx *as_ctx(flowx_ctx *ctx) { return reinterpret_cast<Ctx *>(ctx); }

int check_scene(Ctx *c, int scene)
{
  if (!c->batch) return c->fail(FLOWX_ERR_STATE, "not a batched context: call flowx_batch_set_scenes first");
  if (scene < 0 || scene >= (int)c->segs.size())
    return c->fail(FLOWX_ERR_ARG, "scene index " + std::to_string(scene) + " out of range");
  return FLOWX_OK;
}

int batch_ready(Ctx *c)
{
  if (!c->batch) return c->fail(FLOWX_ERR_STATE, "not a batched context: call flowx_batch_set_scenes first");
  for (size_t s = 0; s < c->segs.size(); ++s)
    if (c->segs[s].voxel > 0.0f && !c->scene_collider[s])
      return c->fail(FLOWX_ERR_STATE, "scene " + std::to_string(s) + " names a collider but none is installed");
  return FLOWX_OK;
}

// Per-particle state saved around autotuning trials.
struct Snapshot {
  float4 *f4[6] = {};
  float2 *lam = nullptr;
  uint32_t *u32[3] = {};
  int pred_idx = 0;
  bool normal_zero = true, normal_in_order = true, delta_in_order = true;
};

int snapshot(Ctx *c, Snapshot &s, bool save)
{
  const size_t n = (size_t)std::max(c->total_particles, 1);
  const size_t cells = (size_t)c->d.cells + 1;
  float4 *live4[6] = {c->d.pos, c->d.vel, c->d.pred_a, c->d.pred_b, c->d.normal, c->d.delta};
  uint32_t *live32[3] = {c->d.ids, c->d.keys, c->d.offsets};
  const size_t len32[3] = {n, n, cells};
  cudaError_t e = cudaSuccess;
  if (save) {
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) e = cudaMalloc((void **)&s.f4[k], n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s.lam, n * sizeof(float2));
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaMalloc((void **)&s.u32[k], len32[k] * 4);
    if (e != cudaSuccess) return c->cuda(e, "autotune snapshot allocation");
    s.pred_idx = c->pred_idx;
    s.normal_zero = c->normal_zero;
    s.normal_in_order = c->normal_in_order;
    s.delta_in_order = c->delta_in_order;
  } else {
    c->next_normals_valid = false;  // the pending normals describe the state being replaced
    c->pred_idx = s.pred_idx;
    c->normal_zero = s.normal_zero;
    c->normal_in_order = s.normal_in_order;
    c->delta_in_order = s.delta_in_order;
  }
  for (int k = 0; k < 6 && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(save ? s.f4[k] : live4[k], save ? live4[k] : s.f4[k], n * sizeof(float4),
                        cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(save ? s.lam : c->d.lam, save ? c->d.lam : s.lam, n * sizeof(float2),
                        cudaMemcpyDeviceToDevice, c->stream);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(save ? s.u32[k] : live32[k], save ? live32[k] : s.u32[k], len32[k] * 4,
                        cudaMemcpyDeviceToDevice, c->stream);
  return c->cuda(e, "autotune snapshot copy");
}

void release(Snapshot &s)
{
  for (auto *p : s.f4)
    if (p) cudaFree(p);
  if (s.lam) cudaFree(s.lam);
  for (auto *p : s.u32)
    if (p) cudaFree(p);
}

}  // namespace

extern "C" {

int flowx_batch_set_scenes(flowx_ctx *ctx, const flowx_push *pushes, int nscenes)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  cudaSetDevice(c->device);
  if (!pushes || nscenes < 1) return c->fail(FLOWX_ERR_ARG, "need at least one scene");
  if (c->flags & FLOWX_FLAG_REFERENCE_ORDER)
    return c->fail(FLOWX_ERR_ARG, "FLOWX_FLAG_REFERENCE_ORDER is for single-scene contexts");
  std::vector<SegParams> segs(nscenes);
  std::vector<long long> voxels(nscenes, 0);
  long long particles = 0, cells = 0, vox = 0;
  for (int k = 0; k < nscenes; ++k) {
    const flowx_push &p = pushes[k];
    const long long sc = (long long)p.i_grid[0] * p.i_grid[1] * p.i_grid[2];
    if (p.i_layout[0] < 0 || p.i_grid[0] <= 0 || p.i_grid[1] <= 0 || p.i_grid[2] <= 0 || sc != p.i_grid[3] ||
        !(p.f_lo[3] > 0.0f))
      return c->fail(FLOWX_ERR_ARG, "scene " + std::to_string(k) + ": inconsistent particle count or grid");
    SegParams &s = segs[k];
    s = SegParams{};
    seg_from_push(p, s);
    s.p_begin = (int)particles;
    s.c_begin = (int)cells;
    s.col_begin = vox;
    if (s.voxel > 0.0f) {
      voxels[k] = (long long)p.i_collider[0] * p.i_collider[1] * p.i_collider[2];
      if (p.i_collider[0] <= 0 || p.i_collider[1] <= 0 || p.i_collider[2] <= 0)
        return c->fail(FLOWX_ERR_ARG, "scene " + std::to_string(k) + ": collider dims must be positive");
    }
    particles += p.i_layout[0];
    cells += sc;
    vox += voxels[k];
  }
  if (particles != c->total_particles)
    return c->fail(FLOWX_ERR_ARG, "scene particle counts sum to " + std::to_string(particles) +
                                      ", the context holds " + std::to_string(c->total_particles));
  if (cells > c->cap_cells) return c->fail(FLOWX_ERR_CAPACITY, "scene cells exceed max_cells");
  if (vox > c->cap_voxels) return c->fail(FLOWX_ERR_CAPACITY, "scene collider voxels exceed max_collider_voxels");
  const bool changed = !c->batch || c->segs.size() != segs.size();
  c->batch = true;
  c->scene_voxels = voxels;
  if (changed) c->scene_collider.assign(nscenes, 0);
  int rc = c->upload_segs(segs, (int)cells);
  if (rc) return rc;
  c->drop_graphs();
  return c->cuda(cudaStreamSynchronize(c->stream), "segment table upload");
}

int flowx_batch_scene_range(flowx_ctx *ctx, int scene, int32_t *first_particle, int32_t *particle_count,
                            int32_t *first_cell, int32_t *cell_count)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  int rc = check_scene(c, scene);
  if (rc) return rc;
  const SegParams &s = c->segs[scene];
  if (first_particle) *first_particle = s.p_begin;
  if (particle_count) *particle_count = s.p_count;
  if (first_cell) *first_cell = s.c_begin;
  if (cell_count) *cell_count = s.c_count;
  return FLOWX_OK;
}

int flowx_batch_set_collider(flowx_ctx *ctx, int scene, const uint8_t *occupancy, const int32_t dims[3],
                             float voxel_size)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  cudaSetDevice(c->device);
  int rc = check_scene(c, scene);
  if (rc) return rc;
  const SegParams &s = c->segs[scene];
  if (!occupancy || !dims) return c->fail(FLOWX_ERR_ARG, "collider occupancy and dims are required");
  if (!(s.voxel > 0.0f)) return c->fail(FLOWX_ERR_STATE, "the scene's push block names no collider");
  if (dims[0] != s.col_nx || dims[1] != s.col_ny || dims[2] != s.col_nz || voxel_size != s.voxel)
    return c->fail(FLOWX_ERR_ARG, "collider dims / voxel differ from the scene's push block");
  rc = c->cuda(cudaMemcpyAsync(c->d.collider + s.col_begin, occupancy, (size_t)c->scene_voxels[scene],
                               cudaMemcpyHostToDevice, c->stream),
               "collider upload");
  if (rc) return rc;
  c->scene_collider[scene] = 1;
  return c->cuda(cudaStreamSynchronize(c->stream), "collider upload");
}

int flowx_batch_build_grid(flowx_ctx *ctx)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  cudaSetDevice(c->device);
  int rc = batch_ready(c);
  if (rc) return rc;
  return c->build_grid_generic();
}

int flowx_batch_substep(flowx_ctx *ctx, int iterations)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  cudaSetDevice(c->device);
  if (iterations < 0 || iterations > 1000) return c->fail(FLOWX_ERR_ARG, "iterations must be in [0, 1000]");
  int rc = batch_ready(c);
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  return c->substep(iterations);
}

int flowx_batch_step(flowx_ctx *ctx, int iterations, int substeps)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  cudaSetDevice(c->device);
  if (iterations < 0 || iterations > 1000) return c->fail(FLOWX_ERR_ARG, "iterations must be in [0, 1000]");
  if (substeps < 1 || substeps > 1000) return c->fail(FLOWX_ERR_ARG, "substeps must be in [1, 1000]");
  int rc = batch_ready(c);
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  return c->step(iterations, substeps);
}

int flowx_batch_splat(flowx_ctx *ctx, int scene, const flowx_push *splat_push, float *host_out, size_t bytes)
{
  if (!ctx || !splat_push) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  cudaSetDevice(c->device);
  int rc = check_scene(c, scene);
  if (rc) return rc;
  const int dims[3] = {splat_push->i_sort[0], splat_push->i_sort[1], splat_push->i_sort[2]};
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return c->fail(FLOWX_ERR_ARG, "splat sample dims must be > 0");
  const long long samples = (long long)dims[0] * dims[1] * dims[2];
  if (samples > c->cap_samples) return c->fail(FLOWX_ERR_CAPACITY, "splat grid larger than max_surface_samples");
  if (host_out && bytes != (size_t)samples * 4) return c->fail(FLOWX_ERR_ARG, "splat output must be samples * 4 bytes");
  rc = batch_ready(c);
  if (rc) return rc;
  rc = c->ensure_grid();
  if (rc) return rc;
  launch_splat_segment(c->d, scene, c->segs[scene].c_begin, c->segs[scene].c_count, splat_push->f_hi,
                       bits_to_float(splat_push->i_sort[3]), splat_push->f_sph[0], splat_push->f_sph[1],
                       splat_push->f_sph[2], dims, c->d.surface, c->stream);
  g_launches += 2;
  rc = c->check_launch("flowx_batch_splat");
  if (rc) return rc;
  if (host_out) {
    rc = c->cuda(cudaMemcpyAsync(host_out, c->d.surface, bytes, cudaMemcpyDeviceToHost, c->stream), "splat download");
    if (rc) return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "splat download");
  }
  return FLOWX_OK;
}

// Block sizes per kernel, chosen by timing the fused substep launch by launch
// with each candidate size on the context's current state (restored after
// every trial, so tuning leaves the simulation where it was).
int flowx_autotune(flowx_ctx *ctx, const flowx_push *push, int iterations, int32_t *chosen)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  cudaSetDevice(c->device);
  if (iterations < 0 || iterations > 1000) return c->fail(FLOWX_ERR_ARG, "iterations must be in [0, 1000]");
  int rc = FLOWX_OK;
  if (c->batch) {
    rc = batch_ready(c);
  } else {
    rc = c->set_push(push);
  }
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  rc = c->ensure_grid();
  if (rc) return rc;
  static const KernelId tunable[] = {K_NORMAL,      K_PREDICT_KEY, K_SCATTER,     K_CELL_SORT_SMALL,
                                     K_PERMUTE_STEP, K_LAMBDA,     K_DELTA_APPLY, K_XSPH_FINALIZE};
  static const int candidates[] = {64, 128, 256, 512};
  const int ncand = (int)(sizeof(candidates) / sizeof(candidates[0]));
  std::vector<std::vector<float>> times(K_COUNT, std::vector<float>(ncand, 0.0f));
  Snapshot snap;
  rc = snapshot(c, snap, true);
  if (rc) {
    release(snap);
    return rc;
  }
  int before[K_COUNT];
  std::memcpy(before, c->d.block, sizeof(before));
  for (int t = 0; t < ncand && rc == FLOWX_OK; ++t) {
    for (KernelId k : tunable) c->d.block[k] = candidates[t];
    for (int rep = 0; rep < 2 && rc == FLOWX_OK; ++rep) {
      std::vector<float> ms(K_COUNT, 0.0f);
      std::vector<int32_t> cnt(K_COUNT, 0);
      rc = c->profile_substeps(iterations, 1, ms.data(), cnt.data());
      if (rep == 1)
        for (KernelId k : tunable) times[k][t] = ms[k];  // second repetition: warm caches
      if (rc == FLOWX_OK) rc = snapshot(c, snap, false);
    }
  }
  if (rc == FLOWX_OK) rc = c->cuda(cudaStreamSynchronize(c->stream), "autotune");
  release(snap);
  c->next_normals_valid = false;  // the restored state is not the one the last trial's normals describe
  if (rc) {
    std::memcpy(c->d.block, before, sizeof(before));
    return rc;
  }
  for (KernelId k : tunable) {
    int best = 0;
    for (int t = 1; t < ncand; ++t)
      if (times[k][t] < times[k][best]) best = t;
    c->d.block[k] = candidates[best];
  }
  c->drop_graphs();
  if (chosen)
    for (int k = 0; k < K_COUNT; ++k) chosen[k] = c->d.block[k];
  return FLOWX_OK;
}

int flowx_set_block_sizes(flowx_ctx *ctx, const int32_t *blocks)
{
  if (!ctx || !blocks) return FLOWX_ERR_ARG;
  Ctx *c = as_ctx(ctx);
  for (int k = 0; k < K_COUNT; ++k) {
    if (blocks[k] < 0 || blocks[k] > 1024 || (blocks[k] % 32) != 0)
      return c->fail(FLOWX_ERR_ARG, "block sizes must be 0 (default) or a multiple of 32 up to 1024");
  }
  for (int k = 0; k < K_COUNT; ++k) c->d.block[k] = blocks[k];
  c->drop_graphs();
  return FLOWX_OK;
}

}  // extern "C"
