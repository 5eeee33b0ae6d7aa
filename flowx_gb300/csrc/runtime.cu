// Host runtime of libflowx: contexts, buffers, the C ABI of include/flowx.h.
//
// A context owns every device buffer of one simulation (or one batch of
// scenes: see batch.cu), a CUDA stream and the CUDA graphs captured for
// flowx_step(). Particle state lives on the device in grid order (see
// flowx_internal.cuh); uploads and downloads convert to and from the
// reference's id-indexed layouts.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>
#include <atomic>
#include <mutex>

#include "../../include/flowx.h"
#include "flowx_internal.cuh"
#include "runtime.h"

using namespace flowx;

namespace flowx {

std::atomic<long long> g_launches{0};
static thread_local std::string g_create_error;

static const char *kKernelNames[K_COUNT] = {
    "normal",        "predict_key",  "scan_reduce", "scan_top",     "scan_down",    "scatter",
    "cell_sort_small", "cell_sort_large", "permute_step", "lambda",  "delta_apply",  "xsph_finalize",
    "splat",         "predict",      "delta",       "apply_delta",  "velocity",     "xsph",
    "finalize",      "permute_all",  "gather",      "scatter_ids",  "voxelize",     "bitonic_sort",
    "row_bounds",
};

// Slices of the constant copy of the segment table, per device: a batch
// context reserves one entry per scene; none left, it reads the device table.
static std::mutex g_cseg_mu;
static std::map<int, std::vector<char>> g_cseg_used;

static int cseg_reserve(int dev, int n)
{
  std::lock_guard<std::mutex> lk(g_cseg_mu);
  auto &used = g_cseg_used[dev];
  if (used.empty()) used.assign(kConstSegs, 0);
  for (int b = 0; b + n <= kConstSegs; ++b) {
    int k = 0;
    while (k < n && !used[b + k]) ++k;
    if (k == n) {
      for (int j = 0; j < n; ++j) used[b + j] = 1;
      return b;
    }
    b += k;
  }
  return -1;
}

static void cseg_release(int dev, int base, int n)
{
  if (base < 0 || n <= 0) return;
  std::lock_guard<std::mutex> lk(g_cseg_mu);
  auto &used = g_cseg_used[dev];
  for (int j = 0; j < n && base + j < (int)used.size(); ++j) used[base + j] = 0;
}

int kernel_max_threads(const void *kernel)
{
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(dev, kernel);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  cudaFuncAttributes attr{};
  int m = 1024;
  if (cudaFuncGetAttributes(&attr, kernel) == cudaSuccess) m = attr.maxThreadsPerBlock;
  cache[key] = m;
  return m;
}

float bits_to_float(int32_t b)
{
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

// Host-side constants of one segment, in float32 and in the order the
// reference's shader code evaluates them (sph_common.glsl:68-81,
// sph_predict.glsl:47, sph_delta.glsl:39).
void seg_from_push(const flowx_push &p, SegParams &s)
{
  const float PI_F = 3.14159265358979323846f;
  s.p_count = p.i_layout[0];
  s.nx = p.i_grid[0];
  s.ny = p.i_grid[1];
  s.nz = p.i_grid[2];
  s.c_count = p.i_grid[3];
  s.lox = p.f_lo[0];
  s.loy = p.f_lo[1];
  s.loz = p.f_lo[2];
  s.cell = p.f_lo[3];
  s.hix = p.f_hi[0];
  s.hiy = p.f_hi[1];
  s.hiz = p.f_hi[2];
  s.radius = p.f_hi[3];
  s.h = p.f_sph[0];
  s.h2 = s.h * s.h;
  s.mass = p.f_sph[1];
  s.rest = p.f_sph[2];
  s.eps = p.f_sph[3];
  s.visc = p.f_sim[0];
  s.dt = p.f_sim[1];
  s.gravity = p.f_sim[2];
  s.damping = p.f_sim[3];
  s.dtc = std::fmax(s.dt, 1e-6f);
  s.scorr_k = bits_to_float(p.i_sort[2]);
  s.sigma = bits_to_float(p.i_sort[3]);
  s.poly6 = 315.0f / (64.0f * PI_F * powf(s.h, 9.0f));
  s.poly6m6 = s.poly6 * -6.0f;
  s.spiky = -45.0f / (PI_F * powf(s.h, 6.0f));
  s.visclap = 45.0f / (PI_F * powf(s.h, 6.0f));
  {
    const float q = 0.2f * s.h;
    const float r2 = q * q;
    if (r2 >= s.h2) {
      s.w_q = 0.0f;
    } else {
      const float d = s.h2 - r2;
      s.w_q = s.poly6 * d * d * d;
    }
  }
  s.v_max = 0.4f * s.h / std::fmax(s.dt, 1e-6f);
  s.mass_spiky = s.mass * s.spiky;
  s.mass_poly6 = s.mass * s.poly6;
  s.poly6_over_wq = s.w_q > 1e-9f ? s.poly6 / s.w_q : 0.0f;
  s.col_nx = p.i_collider[0];
  s.col_ny = p.i_collider[1];
  s.col_nz = p.i_collider[2];
  s.voxel = bits_to_float(p.i_collider[3]);
}

// ---------------------------------------------------------------- helpers
int Ctx::fail(int code, const std::string &msg)
{
  err = msg;
  return code;
}

int Ctx::cuda(cudaError_t e, const char *what)
{
  if (e == cudaSuccess) return FLOWX_OK;
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return FLOWX_ERR_CUDA;
}

int Ctx::check_launch(const char *what)
{
  return cuda(cudaGetLastError(), what);
}

template <class T>
static cudaError_t dalloc(T **p, size_t count)
{
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
  if (e == cudaSuccess) e = cudaMemset(*p, 0, sizeof(T) * count);
  return e;
}

int Ctx::allocate()
{
  const size_t n = (size_t)std::max(total_particles, 1);
  const size_t c = (size_t)std::max(cap_cells, 1);
  cudaError_t e = cudaSuccess;
#define FLOWX_ALLOC(ptr, count) \
  if (e == cudaSuccess) e = dalloc(&(ptr), (count));
  FLOWX_ALLOC(d.pos, n) FLOWX_ALLOC(d.pos_alt, n) FLOWX_ALLOC(d.vel, n) FLOWX_ALLOC(d.vel_alt, n)
  FLOWX_ALLOC(d.pred_a, n) FLOWX_ALLOC(d.pred_b, n) FLOWX_ALLOC(d.normal, n) FLOWX_ALLOC(d.normal_alt, n)
  FLOWX_ALLOC(d.delta, n) FLOWX_ALLOC(d.delta_alt, n) FLOWX_ALLOC(d.lam, n) FLOWX_ALLOC(d.lam_alt, n)
  FLOWX_ALLOC(d.stage, n) FLOWX_ALLOC(d.keys, n) FLOWX_ALLOC(d.ids, n) FLOWX_ALLOC(d.key_tmp, n)
  FLOWX_ALLOC(d.rank_tmp, n) FLOWX_ALLOC(d.pairs, n) FLOWX_ALLOC(d.pairs_tmp, n)
  FLOWX_ALLOC(d.counts, c) FLOWX_ALLOC(d.offsets, c + 1) FLOWX_ALLOC(d.block_sums, c / 2048 + 2)
  FLOWX_ALLOC(d.big_cells, c + 1) FLOWX_ALLOC(d.collider, (size_t)std::max<long long>(cap_voxels, 1))
  FLOWX_ALLOC(d.surface, (size_t)std::max<long long>(cap_samples, 1))
  FLOWX_ALLOC(d_segs, (size_t)std::max<int>((int)segs.size(), 1))
  FLOWX_ALLOC(d_src_slot, n)
  FLOWX_ALLOC(d.row_masks, n * 9) FLOWX_ALLOC(d.row_wide, n) FLOWX_ALLOC(d.cell_lo, c) FLOWX_ALLOC(d.cell_hi, c)
  FLOWX_ALLOC(d.quads, (n + 3) / 4) FLOWX_ALLOC(d.plam, n) FLOWX_ALLOC(d.xv, n) FLOWX_ALLOC(d.slot_seg, n)
  FLOWX_ALLOC(d.quad_bounds, (n + 3) / 4) FLOWX_ALLOC(d.row_yz, c) FLOWX_ALLOC(d.sort_x, n)
  FLOWX_ALLOC(d.quads_alt, (n + 3) / 4)
  if (flags & FLOWX_FLAG_REFERENCE_ORDER) {
    // solver/sph.py's sorted_count: the next power of two >= N, at least 2
    size_t S = 2;
    while (S < (size_t)total_particles) S <<= 1;
    d.bitonic_n = (int)S;
    FLOWX_ALLOC(d.bitonic, S) FLOWX_ALLOC(d.bitonic_inv, n)
  }
#undef FLOWX_ALLOC
  if (e != cudaSuccess) return cuda(e, "device allocation");
  d.segs = d_segs;
  d.nseg = (int)segs.size();
  d.cseg_base = -1;
  d.n = total_particles;
  d.cells = 0;
  d.warp_passes = (flags & FLOWX_FLAG_WARP_PASSES) ? 1
                  : (flags & FLOWX_FLAG_THREAD_PASSES) ? 0
                  : (total_particles <= FLOWX_WARP_PASSES_MAX_PARTICLES ? 1 : 0);
  d.trim = 0;  // set with the segment table (upload_segs)
  d.x_order = 0;
  // ids start as the identity: slot k holds particle k.
  std::vector<uint32_t> ident(n);
  for (size_t k = 0; k < n; ++k) ident[k] = (uint32_t)k;
  e = cudaMemcpy(d.ids, ident.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice);
  return cuda(e, "ids init");
}

void Ctx::release()
{
  cseg_release(device, d.cseg_base, cseg_count);
  d.cseg_base = -1;
  cseg_count = 0;
  for (auto &kv : graphs) {
    cudaGraphExecDestroy(kv.second.exec);
  }
  graphs.clear();
  void *ptrs[] = {d.pos,    d.pos_alt, d.vel,       d.vel_alt,  d.pred_a,   d.pred_b,  d.normal,     d.normal_alt,
                  d.delta,  d.delta_alt, d.lam,     d.lam_alt,  d.stage,    d.keys,    d.ids,        d.key_tmp,
                  d.rank_tmp, d.pairs, d.pairs_tmp, d.counts,   d.offsets,  d.block_sums, d.big_cells, d.collider,
                  d.surface, d_segs,   d_src_slot,  d_prims,  d_mesh,  d.row_masks, d.row_wide, d.cell_lo, d.cell_hi, d.quads, d.plam, d.xv, d.slot_seg,
                  d.bitonic, d.bitonic_inv, d.quad_bounds, d.row_yz, d.sort_x, d.quads_alt,
                  d.chunk_masks, d.chunk_base};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (stream) cudaStreamDestroy(stream);
  for (auto &ev : events) cudaEventDestroy(ev);
  events.clear();
  stream = nullptr;
}

float4 *Ctx::pred_cur() { return pred_idx == 0 ? d.pred_a : d.pred_b; }

// Captured graphs bake in launch shapes; drop them when those change.
void Ctx::drop_graphs()
{
  for (auto &kv : graphs) cudaGraphExecDestroy(kv.second.exec);
  graphs.clear();
}

// Resolve and upload the segment table for a push (single-scene contexts).
int Ctx::set_push(const flowx_push *push)
{
  if (!push) return fail(FLOWX_ERR_ARG, "push block is NULL");
  if (batch) return fail(FLOWX_ERR_STATE, "batched context: use the flowx_batch_* entry points");
  if (push->i_layout[0] != total_particles)
    return fail(FLOWX_ERR_ARG, "push i_layout.x (particle count " + std::to_string(push->i_layout[0]) +
                                   ") differs from the context's " + std::to_string(total_particles));
  const long long cells = (long long)push->i_grid[0] * push->i_grid[1] * push->i_grid[2];
  if (push->i_grid[0] <= 0 || push->i_grid[1] <= 0 || push->i_grid[2] <= 0 || cells != push->i_grid[3])
    return fail(FLOWX_ERR_ARG, "push i_grid is inconsistent (cells_x * cells_y * cells_z != cell_count)");
  if (cells > cap_cells)
    return fail(FLOWX_ERR_CAPACITY, "cell_count " + std::to_string(cells) + " exceeds the context's max_cells " +
                                        std::to_string(cap_cells));
  if (!(push->f_lo[3] > 0.0f)) return fail(FLOWX_ERR_ARG, "cell size must be > 0");
  SegParams s{};
  seg_from_push(*push, s);
  s.p_begin = 0;
  s.c_begin = 0;
  s.col_begin = 0;
  if (s.voxel > 0.0f) {
    if (!collider_installed)
      return fail(FLOWX_ERR_STATE, "push names a collider (voxel > 0) but none is installed");
    if (s.col_nx != collider_dims[0] || s.col_ny != collider_dims[1] || s.col_nz != collider_dims[2])
      return fail(FLOWX_ERR_ARG, "push i_collider dims differ from the installed collider grid");
  }
  return upload_segs({s}, (int)cells);
}

int Ctx::upload_segs(const std::vector<SegParams> &s_in, int cells)
{
  // number the x-rows (cells of one (y, z)) of the segments consecutively
  std::vector<SegParams> s = s_in;
  int xrows = 0;
  for (auto &q : s) {
    q.r_begin = xrows;
    xrows += q.ny * q.nz;
  }
  const bool same = s.size() == segs.size() && std::memcmp(s.data(), segs.data(), s.size() * sizeof(SegParams)) == 0;
  if (!same || cells != d.cells) next_normals_valid = false;  // reach or geometry changed
  if (!same || !segs_uploaded) {
    if (s.size() > seg_capacity) {
      // A batch with more scenes than the table holds: grow it (stream work
      // that may still read the old table is finished first).
      int rc = cuda(cudaStreamSynchronize(stream), "segment table resize");
      if (rc) return rc;
      if (d_segs) cudaFree(d_segs);
      d_segs = nullptr;
      rc = cuda(cudaMalloc((void **)&d_segs, s.size() * sizeof(SegParams)), "segment table allocation");
      if (rc) return rc;
      seg_capacity = s.size();
      drop_graphs();
    }
    segs = s;
    int rc = cuda(cudaMemcpyAsync(d_segs, segs.data(), segs.size() * sizeof(SegParams), cudaMemcpyHostToDevice,
                                  stream),
                  "segment table upload");
    if (rc) return rc;
    if (segs.size() > 1) {
      // slot -> segment (the pageable copy is staged before this returns)
      std::vector<int32_t> owner((size_t)total_particles, 0);
      for (size_t k = 0; k < segs.size(); ++k)
        for (int q = 0; q < segs[k].p_count; ++q) {
          const long long slot = (long long)segs[k].p_begin + q;
          if (slot >= 0 && slot < total_particles) owner[(size_t)slot] = (int32_t)k;
        }
      rc = cuda(cudaMemcpyAsync(d.slot_seg, owner.data(), owner.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                stream),
                "slot segment table upload");
      if (rc) return rc;
    }
    segs_uploaded = true;
    d.segs = d_segs;
    d.nseg = (int)segs.size();
    d.seg0 = segs.empty() ? SegParams{} : segs[0];
    // Cells coarser than the reach (1.5 h or more): the thread-per-particle
    // neighbour passes trim each stencil row to the particle's reach
    // (for_each_within_trimmed_staged); cells of h keep the untrimmed walk. The
    // re-associated arithmetic orders each cell by x, which makes the trimmed
    // runs short and, on cells of h, gives a warp's lanes more alike
    // neighbourhoods (0.6% per frame on the 4M workload); the reference's
    // expressions keep the (cell, id) order the oracle runs, and the
    // reference's network keeps its own.
    bool coarse = false;
    for (const auto &q : segs) coarse = coarse || q.cell >= 1.5f * q.h;
    d.trim = (coarse && !d.warp_passes) ? 1 : 0;
    if (d.trim && !d.chunk_masks) {  // the trimmed walk's chunk record, on first use
      const size_t n = (size_t)std::max(total_particles, 1) * kMaxChunks;
      cudaError_t e = dalloc(&d.chunk_masks, n);
      if (e == cudaSuccess) e = dalloc(&d.chunk_base, n);
      if (e != cudaSuccess) return cuda(e, "chunk record allocation");
    }
    d.x_order = (flags & (FLOWX_FLAG_EXACT | FLOWX_FLAG_REFERENCE_ORDER)) ? 0 : 1;
    if (segs.size() > 1) {
      const int need = (int)segs.size();
      if (need > cseg_count) {
        cseg_release(device, d.cseg_base, cseg_count);
        d.cseg_base = cseg_reserve(device, need);
        cseg_count = d.cseg_base >= 0 ? need : 0;
      }
      if (d.cseg_base >= 0) {
        cudaError_t e = const_segs_upload_pbf(d.cseg_base, segs.data(), need, stream);
        if (e == cudaSuccess) e = const_segs_upload_warp(d.cseg_base, segs.data(), need, stream);
        if (e == cudaSuccess) e = const_segs_upload_grid(d.cseg_base, segs.data(), need, stream);
        if (e != cudaSuccess) return cuda(e, "constant segment table upload");
      }
    }
    drop_graphs();  // their launches carry seg0
    d.xrows = xrows;
  }
  if (cells != d.cells) {
    if (have_grid && cells != d.cells) have_grid = false;
    d.cells = cells;
  }
  return FLOWX_OK;
}

// ------------------------------------------------------------ grid build
// Cell order from the keys and the scan: the counting sort's (cell, id) or
// (cell, predicted x) order, or the reference's own network
// (FLOWX_FLAG_REFERENCE_ORDER).
void Ctx::issue_cell_order(bool x_order)
{
  if (flags & FLOWX_FLAG_REFERENCE_ORDER) {
    g_launches += launch_reference_order(d, stream);
  } else {
    launch_scatter(d, stream, x_order);
    launch_cell_sort(d, stream);
    g_launches += 3;
  }
}

void Ctx::issue_build_from_pred(const float4 *pred)
{
  launch_key_only(d, pred, stream);
  launch_scan(d, stream);
  g_launches += 4;
  issue_cell_order(false);
}

int Ctx::build_grid_generic()
{
  next_normals_valid = false;
  float4 *src = pred_cur();
  float4 *dst = pred_idx == 0 ? d.pred_b : d.pred_a;
  issue_build_from_pred(src);
  launch_permute_all(d, src, dst, stream);
  g_launches += 1;
  const size_t n = (size_t)total_particles;
  cudaError_t e = cudaSuccess;
  if (n) {
    e = cudaMemcpyAsync(d.pos, d.pos_alt, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.vel, d.vel_alt, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d.normal, d.normal_alt, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d.delta, d.delta_alt, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.lam, d.lam_alt, n * sizeof(float2), cudaMemcpyDeviceToDevice, stream);
  }
  if (e != cudaSuccess) return cuda(e, "grid build copy-back");
  pred_idx ^= 1;
  have_grid = true;
  keys_host_valid = false;
  return check_launch("flowx_build_grid");
}

// The fused substep body (see pbf.cu's header for the pass mapping).
// pred_in_idx: predicted buffer holding last substep's corrected predictions.
int Ctx::issue_substep(int iterations, int pred_in_idx, bool normals_ready)
{
  float4 *pred_in = pred_in_idx == 0 ? d.pred_a : d.pred_b;
  const bool sigma = segs_need_normal();
  const bool exact = (flags & FLOWX_FLAG_EXACT) != 0;
  // The substep's normals go to scratch in the old slot order; the permute
  // moves them to the new order in the canonical buffer. The normal pass
  // walks the previous substep's grid; when normals_ready, that substep's
  // XSPH pass already evaluated it there.
  if (sigma && !normals_ready) {
    launch_normal_f(d, pred_in, d.normal_alt, exact, stream);
    g_launches += 1;
  }
  launch_predict_key(d, d.normal_alt, stream);
  launch_scan(d, stream);
  issue_cell_order(d.x_order != 0);
  launch_permute_step(d, d.pred_a, d.normal_alt, stream);
  g_launches += 5;
  float4 *q_in = d.pred_a, *q_out = d.pred_b;
  for (int it = 0; it < iterations; ++it) {
    if (d.trim) {
      launch_row_bounds(d, q_in, stream);
      g_launches += 1;
    }
    launch_lambda_f(d, q_in, exact, stream);
    launch_delta_apply_f(d, q_in, q_out, exact, it == iterations - 1, stream);
    g_launches += 2;
    std::swap(q_in, q_out);
    if (d.trim) std::swap(d.quads, d.quads_alt);  // the quads of q_in, written by that delta_apply
  }
  if (iterations == 0) {
    launch_xsph_inputs(d, q_in, exact, stream);
    g_launches += 1;
  }
  if (d.trim) {
    launch_row_bounds(d, q_in, stream);
    g_launches += 1;
  }
  launch_xsph_finalize_f(d, q_in, d.pos, (flags & FLOWX_FLAG_KEEP_DELTA) != 0, exact, sigma, stream);
  g_launches += 1;
  return FLOWX_OK;
}

// Which buffers a fused substep leaves in the new grid order: positions,
// velocities, predicted and lambda always; normal when the normal pass ran
// (or it holds only the zeros it was created with); delta only with
// FLOWX_FLAG_KEEP_DELTA. The others can no longer be mapped to particle ids.
void Ctx::after_fused_substep()
{
  next_normals_valid = segs_need_normal();
  if (segs_need_normal()) {
    normal_zero = false;
  } else if (!normal_zero) {
    normal_in_order = false;
  }
  delta_in_order = (flags & FLOWX_FLAG_KEEP_DELTA) != 0;
}

bool Ctx::segs_need_normal() const
{
  for (const auto &s : segs)
    if (s.sigma > 0.0f) return true;
  return false;
}

int Ctx::ensure_grid()
{
  if (have_grid) return FLOWX_OK;
  // No grid yet (fresh context or changed cell geometry): build one from the
  // current predictions, as the reference's seed does before the first
  // substep (solver/sph.py:606, :730).
  return build_grid_generic();
}

int Ctx::substep(int iterations)
{
  int rc = ensure_grid();
  if (rc) return rc;
  issue_substep(iterations, pred_idx, next_normals_valid);
  pred_idx = iterations % 2 == 0 ? 0 : 1;
  keys_host_valid = false;
  after_fused_substep();
  return check_launch("flowx_substep");
}

int Ctx::step(int iterations, int substeps)
{
  int rc = ensure_grid();
  if (rc) return rc;
  const int end_idx = iterations % 2 == 0 ? 0 : 1;
  GraphKey key{iterations, substeps, pred_idx, d.cells, segs_need_normal() ? 1 : 0, flags, next_normals_valid ? 1 : 0};
  auto it = graphs.find(key);
  if (it == graphs.end()) {
    cudaGraph_t graph = nullptr;
    rc = cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
    if (rc) return rc;
    const long long before = g_launches.load();
    int idx = pred_idx;
    for (int s = 0; s < substeps; ++s) {
      issue_substep(iterations, idx, s > 0 || next_normals_valid);
      idx = end_idx;
    }
    const long long kernels = g_launches.load() - before;
    g_launches -= kernels;  // captured, not launched
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
    if (e != cudaSuccess) return cuda(e, "graph capture end");
    GraphEntry entry{};
    entry.kernels = kernels;
    e = cudaGraphInstantiate(&entry.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda(e, "graph instantiate");
    it = graphs.emplace(key, entry).first;
  }
  rc = cuda(cudaGraphLaunch(it->second.exec, stream), "graph launch");
  if (rc) return rc;
  g_launches += it->second.kernels;
  pred_idx = end_idx;
  keys_host_valid = false;
  after_fused_substep();
  return FLOWX_OK;
}

}  // namespace flowx

// ------------------------------------------------------------ C ABI
extern "C" {

int flowx_create(const flowx_config *config, flowx_ctx **out)
{
  if (!config || !out) {
    g_create_error = "flowx_create: config and out must not be NULL";
    return FLOWX_ERR_ARG;
  }
  *out = nullptr;
  if (config->particle_count < 0 || config->max_cells < 1 || config->max_collider_voxels < 0 ||
      config->max_surface_samples < 0) {
    g_create_error = "flowx_create: negative particle count or capacity, or max_cells < 1";
    return FLOWX_ERR_ARG;
  }
  if (config->flags & ~(FLOWX_FLAG_KEEP_DELTA | FLOWX_FLAG_EXACT | FLOWX_FLAG_REFERENCE_ORDER |
                        FLOWX_FLAG_WARP_PASSES | FLOWX_FLAG_THREAD_PASSES)) {
    g_create_error = "flowx_create: unknown bits in flags";
    return FLOWX_ERR_ARG;
  }
  if ((config->flags & FLOWX_FLAG_WARP_PASSES) && (config->flags & FLOWX_FLAG_THREAD_PASSES)) {
    g_create_error = "flowx_create: FLOWX_FLAG_WARP_PASSES and FLOWX_FLAG_THREAD_PASSES exclude each other";
    return FLOWX_ERR_ARG;
  }
  if (config->particle_count > (1 << 24)) {
    g_create_error = "flowx_create: particle_count above 2^24 cannot be represented in the reference's "
                     "float-coded key buffer";
    return FLOWX_ERR_CAPACITY;
  }
  Ctx *c = new Ctx();
  c->device = config->device;
  c->flags = config->flags;
  c->total_particles = config->particle_count;
  c->cap_cells = config->max_cells;
  c->cap_voxels = config->max_collider_voxels;
  c->cap_samples = config->max_surface_samples;
  SegParams s{};
  s.p_begin = 0;
  s.p_count = config->particle_count;
  c->segs = {s};
  int rc = c->init_device();
  if (rc) {
    g_create_error = c->err;
    c->release();
    delete c;
    return rc;
  }
  *out = reinterpret_cast<flowx_ctx *>(c);
  return FLOWX_OK;
}

int flowx_destroy(flowx_ctx *ctx)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->release();
  delete c;
  return FLOWX_OK;
}

const char *flowx_last_error(const flowx_ctx *ctx)
{
  if (!ctx) return g_create_error.c_str();
  return reinterpret_cast<const Ctx *>(ctx)->err.c_str();
}

int flowx_synchronize(flowx_ctx *ctx)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  return c->cuda(cudaStreamSynchronize(c->stream), "stream synchronize");
}

int flowx_get_stream(flowx_ctx *ctx, void **stream)
{
  if (!ctx || !stream) return FLOWX_ERR_ARG;
  *stream = (void *)reinterpret_cast<Ctx *>(ctx)->stream;
  return FLOWX_OK;
}

int flowx_build_grid(flowx_ctx *ctx, const flowx_push *push)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  int rc = c->set_push(push);
  if (rc) return rc;
  return c->build_grid_generic();
}

int flowx_substep(flowx_ctx *ctx, const flowx_push *push, int iterations)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  if (iterations < 0 || iterations > 1000) return c->fail(FLOWX_ERR_ARG, "iterations must be in [0, 1000]");
  cudaSetDevice(c->device);
  int rc = c->set_push(push);
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  return c->substep(iterations);
}

int flowx_step(flowx_ctx *ctx, const flowx_push *push, int iterations, int substeps)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  if (iterations < 0 || iterations > 1000) return c->fail(FLOWX_ERR_ARG, "iterations must be in [0, 1000]");
  if (substeps < 1 || substeps > 1000) return c->fail(FLOWX_ERR_ARG, "substeps must be in [1, 1000]");
  cudaSetDevice(c->device);
  int rc = c->set_push(push);
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  return c->step(iterations, substeps);
}

int flowx_run_pass(flowx_ctx *ctx, int pass_id, const flowx_push *push)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  int rc = c->set_push(push);
  if (rc) return rc;
  rc = c->ensure_offsets();
  if (rc) return rc;
  const DeviceState &d = c->d;
  float4 *pred = c->pred_cur();
  const bool needs_grid = pass_id == FLOWX_PASS_NORMAL || pass_id == FLOWX_PASS_LAMBDA ||
                          pass_id == FLOWX_PASS_DELTA || pass_id == FLOWX_PASS_XSPH;
  if (needs_grid && !c->have_grid)
    return c->fail(FLOWX_ERR_STATE, "neighbour pass before any grid build: call flowx_build_grid first");
  c->next_normals_valid = false;
  switch (pass_id) {
    case FLOWX_PASS_NORMAL:
      launch_normal(d, pred, d.normal, c->stream);
      c->normal_in_order = true;
      c->normal_zero = false;
      break;
    case FLOWX_PASS_PREDICT: launch_predict(d, pred, c->stream); break;
    case FLOWX_PASS_LAMBDA:
      launch_lambda(d, pred, c->stream);  // with the quads' fill and, trimming, the row bounds
      g_launches += 1 + (d.trim ? 1 : 0);
      break;
    case FLOWX_PASS_DELTA:
      launch_delta(d, pred, c->stream);
      c->delta_in_order = true;
      break;
    case FLOWX_PASS_APPLY_DELTA: launch_apply(d, pred, c->stream); break;
    case FLOWX_PASS_VELOCITY: launch_velocity(d, pred, c->stream); break;
    case FLOWX_PASS_XSPH:
      launch_xsph(d, pred, c->stream);
      c->delta_in_order = true;
      break;
    case FLOWX_PASS_FINALIZE: launch_finalize(d, pred, c->stream); break;
    case FLOWX_PASS_GRID_KEY:
    case FLOWX_PASS_SORT:
    case FLOWX_PASS_CELL_CLEAR:
    case FLOWX_PASS_CELL_RANGE:
      return c->fail(FLOWX_ERR_ARG, "grid-key, sort, cell-clear and cell-range run together: use flowx_build_grid");
    default: return c->fail(FLOWX_ERR_ARG, "unknown pass id " + std::to_string(pass_id));
  }
  g_launches += 1;
  return c->check_launch("flowx_run_pass");
}

int flowx_time_steps(flowx_ctx *ctx, const flowx_push *push, int iterations, int substeps, int steps, float *ms)
{
  if (!ctx || !ms || steps < 1) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  int rc = flowx_step(ctx, push, iterations, substeps);
  if (rc) return rc;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, c->stream);
  for (int s = 0; s < steps && rc == FLOWX_OK; ++s) rc = c->step(iterations, substeps);
  cudaEventRecord(b, c->stream);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  return c->check_launch("flowx_time_steps");
}

int flowx_kernel_count(void) { return K_COUNT; }

const char *flowx_kernel_name(int kernel_id)
{
  if (kernel_id < 0 || kernel_id >= K_COUNT) return "";
  return kKernelNames[kernel_id];
}

int64_t flowx_launch_count(void) { return (int64_t)g_launches.load(); }


}  // extern "C"
