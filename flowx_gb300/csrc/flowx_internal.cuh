// Internal declarations shared by the CUDA translation units of libflowx.
//
// Device-side data layout (HBM):
//   particle arrays live in *grid order*: slot k holds the particle whose
//   (cell, id) is the k-th smallest under the last grid build ((cell,
//   predicted x) in the re-associated arithmetic's fused build), so the 3x3x3
//   neighbour stencil of any particle is nine contiguous runs of slots (the
//   three x-adjacent cells of one (y, z) row are adjacent in memory).
//   ids[k] maps a slot back to the caller's particle id; every upload and
//   download goes through that permutation, so callers always see the
//   reference's id-indexed layout (solver/sph.py:127-152).
//
//   float4 pos / vel / pred / normal / delta   (xyz + the reference's w lane)
//   float2 lam                                 (density, lambda)
//   uint32 keys[k]                             (global cell index of slot k)
//   uint32 cell_offset[C + 1]                  (exclusive scan of cell counts:
//                                               cell c owns [off[c], off[c+1]))
//   uint8  collider voxels                     (x fastest, 1 = occupied)
//
// Several independent scenes ("segments") can share one context: their
// particles and cells are concatenated and every kernel looks up its
// segment's parameters in a device table, so one launch per pass serves all
// scenes. A single scene is a table of one segment, whose parameters the
// substep's kernels take from their by-value DeviceState argument instead
// (DeviceState::seg0): the arithmetic then reads them as constant operands,
// with no load and no register (6-11% per neighbour pass on the 4M-particle
// workload). A batch reads them from its slice of a constant-memory copy of
// the table (c_segs) when one is free, through the constant cache instead of
// L1 (3.8% on the 64-scene batched workload); otherwise from the device table.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace flowx {

constexpr int kMaxCellScan = 512;       // shaders/sph_common.glsl:30
constexpr int kMaxColliderSearch = 2;   // shaders/sph_finalize.glsl:13
constexpr int kSurfaceCellRadius = 2;   // shaders/surface_splat.glsl:30
constexpr int kSmallCellSort = 64;      // cells above this go to the block sorter
// Cells above this keep the scatter's order instead of the (cell, id) order:
// the block sorter is quadratic in a cell's size, and such cells only arise
// from degenerate states (e.g. a blown-up run whose NaN positions all map to
// one cell). The key column, cell ranges and membership stay exact; the
// reference's unstable bitonic sort leaves such a cell in arbitrary order too.
constexpr int kMaxRankSortCell = 4096;
// The trimmed walk (cells coarser than the reach) records at most this many
// chunks per slot for the pass that replays them; a slot with more (or a row
// over MAX_CELL_SCAN, walked directly) is marked kChunksNotRecorded and the
// replaying pass walks it again.
constexpr int kMaxChunks = 16;
constexpr uint8_t kChunksNotRecorded = 0xff;

// Per-segment parameters, resolved on the host from the push-constant block
// (shaders/sph_common.glsl:10-17). Kernel constants that depend only on the
// push values (kernel coefficients, speed limit) are computed once on the
// host in float32, in the same operation order as the reference's shader
// code, so the device never re-derives them.
struct SegParams {
  int p_begin, p_count;        // slots [p_begin, p_begin + p_count)
  int c_begin, c_count;        // cells [c_begin, c_begin + c_count)
  int r_begin;                 // first x-row (the nx cells of one (y, z)) in the context's numbering
  int nx, ny, nz;              // i_grid.xyz
  float lox, loy, loz, cell;   // f_lo
  float hix, hiy, hiz, radius; // f_hi (solver passes) / surface lo (splat)
  float h, h2, mass, rest;     // f_sph.x, h*h, f_sph.y, f_sph.z
  float eps;                   // f_sph.w (relaxation)
  float visc, dt, gravity, damping;  // f_sim
  float dtc;                   // max(dt, 1e-6)
  float scorr_k, sigma;        // i_sort.z / .w as floats
  float poly6, poly6m6, spiky, visclap, w_q, v_max;
  // products the re-associated (FAST) pair bodies use, formed once on the host
  float mass_spiky, mass_poly6, poly6_over_wq;
  int col_nx, col_ny, col_nz;  // i_collider.xyz
  float voxel;                 // i_collider.w as float; 0 = no collider
  long long col_begin;         // byte offset of this segment's voxels
  // splat (surface grid) parameters, only read by the splat kernel
  int snx, sny, snz;
  float sspacing;
  long long s_begin;           // first sample of this segment in the output
};

// Kernels whose block size a context may choose (flowx_autotune).
enum KernelId {
  K_NORMAL = 0,
  K_PREDICT_KEY,
  K_SCAN_REDUCE,
  K_SCAN_TOP,
  K_SCAN_DOWN,
  K_SCATTER,
  K_CELL_SORT_SMALL,
  K_CELL_SORT_LARGE,
  K_PERMUTE_STEP,
  K_LAMBDA,
  K_DELTA_APPLY,
  K_XSPH_FINALIZE,
  K_SPLAT,
  K_PREDICT,
  K_DELTA,
  K_APPLY,
  K_VELOCITY,
  K_XSPH,
  K_FINALIZE,
  K_PERMUTE_ALL,
  K_GATHER,
  K_SCATTER_IDS,
  K_VOXELIZE,
  K_BITONIC,
  K_ROW_BOUNDS,
  K_COUNT
};

// Largest block a kernel can be launched with on the current device (its
// register and shared-memory use; cached per kernel).
int kernel_max_threads(const void *kernel);

// Block size for a launch: the context's choice for the kernel (0 = `def`),
// capped at what the kernel can launch with, in whole warps.
#define FLOWX_BLOCK(d, kid, def, kernel)                                                   \
  ([&]() {                                                                                  \
    int b_ = (d).block[kid] > 0 ? (d).block[kid] : (def);                                   \
    const int m_ = kernel_max_threads((const void *)(kernel));                              \
    if (b_ > m_) b_ = m_ & ~31;                                                             \
    return b_ < 32 ? 32 : b_;                                                               \
  }())

// Device pointers of one context's state (all in grid order).
// Predicted positions of four consecutive slots, coordinate-major (slot
// 4g + u in lane u of x, y and z): the candidate filter of the neighbour
// passes reads four candidates with three 16-byte loads and tests them two
// at a time with paired float arithmetic.
struct SlotQuad {
  float4 x, y, z;
};

// Slot k's predicted position into its lane of the slot quads.
__device__ __forceinline__ void store_quad(SlotQuad *__restrict__ quads, int k, float x, float y, float z)
{
  float *g = reinterpret_cast<float *>(quads + (k >> 2));
  const int u = k & 3;
  g[u] = x;
  g[4 + u] = y;
  g[8 + u] = z;
}

struct DeviceState {
  int block[K_COUNT];       // block size per kernel, 0 = the kernel's default
  float4 *pos, *pos_alt;    // positions; pos_alt receives the permuted copy
  float4 *vel, *vel_alt;
  float4 *pred_a, *pred_b;  // predicted positions (Jacobi ping-pong)
  float4 *normal, *normal_alt;
  float4 *delta, *delta_alt;
  float2 *lam, *lam_alt;
  float4 *stage;            // staging for uploads / downloads
  uint32_t *keys, *ids;     // per slot
  uint32_t *key_tmp, *rank_tmp;  // per old slot during a grid build
  unsigned long long *pairs, *pairs_tmp;  // (id << 32 | old slot) per new slot
  uint32_t *counts;         // per cell, zero between builds
  uint32_t *offsets;        // per cell + 1
  uint32_t *block_sums;     // scan scratch
  uint32_t *big_cells;      // [0] = count, then cell indices
  uint8_t *collider;
  float *surface;
  float4 *cell_lo, *cell_hi;  // per cell: bounds of its particles' positions (the splat's cell test)
  unsigned long long *row_masks;  // the lambda pass's neighbour masks, 9 per slot (row-major)
  uint8_t *row_wide;        // per slot: masks not recorded (a row over 64 slots); trimmed walk: the
                            // number of chunks recorded, or kChunksNotRecorded
  unsigned long long *chunk_masks;  // trimmed walk (trim): the lambda pass's non-empty chunk masks,
  uint32_t *chunk_base;             // kMaxChunks per slot (chunk-major), and each one's first slot
  float4 *plam;             // per slot: predicted position and lambda of the last lambda pass
  float4 *xv;               // per slot: velocity (pred - pos) / dt and max(rho, 1e-6) entering XSPH
  SlotQuad *quads;          // ceil(n / 4) groups: the predicted positions the next lambda or
                            // XSPH pass filters (written by permute_step, delta_apply, fill_quads)
  SlotQuad *quads_alt;      // trimmed walk (trim): delta_apply writes the next quads here, since
                            // its own walk reads d.quads; the runtime swaps the two after it
  // Candidate trimming of those passes (row_bounds, before each of them):
  float2 *quad_bounds;      // per quad g: (.x) the largest x of the slots of its x-row from the
                            // x-row's first slot to slot 4g + 3, (.y) the smallest x from slot 4g
                            // to the x-row's last slot
  float4 *row_yz;           // per cell: y and z bounds (ymin, ymax, zmin, zmax) of the particles of
                            // the cells x - 1, x, x + 1 of its x-row
  uint32_t *sort_x;         // per old slot during a fused grid build: its predicted x as an
                            // order-preserving integer (x_order)
  int xrows;                // x-rows of all segments
  int trim;                 // lambda and XSPH trim their rows (quad_bounds, row_yz are maintained)
  int x_order;              // the fused grid build orders each cell by predicted x, not by id
  unsigned long long *bitonic;  // FLOWX_FLAG_REFERENCE_ORDER: the (cell << 32 | id) array the
                                // reference's sort network orders (bitonic_n entries)
  uint32_t *bitonic_inv;    // per particle id: its slot before the build
  int bitonic_n;            // next power of two >= n (the reference's sorted_count)
  const SegParams *segs;
  SegParams seg0;           // segs[0], read from the kernel argument by single-scene launches
  int cseg_base;            // this context's first entry of c_segs, or -1 (not there)
  int32_t *slot_seg;        // per slot: its segment (read only when nseg > 1)
  int nseg;
  int warp_passes;          // neighbour passes one warp per particle (pbf_warp.cu), else one thread
  int n;                    // total particles
  int cells;                // total cells
  int sm_count;             // multiprocessors of the context's device
};

// Segment of slot k. A segment's particles keep its slot range
// [p_begin, p_begin + p_count) through every grid build (its cells are a
// contiguous range holding exactly its particles), so the table is written
// once per segment-table upload.
__device__ __forceinline__ int slot_segment(const DeviceState &d, int k)
{
  return d.nseg == 1 ? 0 : __ldg(&d.slot_seg[k]);
}

// Where a kernel reads its slot's segment parameters: the device table, the
// kernel argument (a single-scene context: seg0), or the context's slice of
// a constant-memory copy of the table (a batch whose table fits it).
enum SegSource { kSegTable = 0, kSegArg = 1, kSegConst = 2 };
constexpr int kConstSegs = 128;
// One copy per translation unit (no relocatable device code); the units that
// launch substep kernels each export an upload (const_segs_upload_*).
static __constant__ SegParams c_segs[kConstSegs];

template <int SEG>
__device__ __forceinline__ const SegParams &slot_params(const DeviceState &d, int k)
{
  if constexpr (SEG == kSegArg)
    return d.seg0;
  else if constexpr (SEG == kSegConst)
    return c_segs[d.cseg_base + slot_segment(d, k)];
  else
    return d.segs[slot_segment(d, k)];
}

inline int seg_source(const DeviceState &d)
{
  return d.nseg == 1 ? kSegArg : (d.cseg_base >= 0 ? kSegConst : kSegTable);
}

// f(std::integral_constant<int, SEG>) for the context's source.
template <class F>
inline void with_seg_source(const DeviceState &d, F &&f)
{
  switch (seg_source(d)) {
    case kSegArg: f(std::integral_constant<int, kSegArg>{}); break;
    case kSegConst: f(std::integral_constant<int, kSegConst>{}); break;
    default: f(std::integral_constant<int, kSegTable>{}); break;
  }
}

// The constant copies of the segment table (entries [base, base + n)).
cudaError_t const_segs_upload_pbf(int base, const SegParams *s, int n, cudaStream_t st);
cudaError_t const_segs_upload_warp(int base, const SegParams *s, int n, cudaStream_t st);
cudaError_t const_segs_upload_grid(int base, const SegParams *s, int n, cudaStream_t st);

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// sph_common.glsl:50-54 (cell_coord) and :56-59 (cell_index), local to the segment.
__device__ __forceinline__ int3 cell_coord(const SegParams &s, float px, float py, float pz)
{
  int3 g;
  g.x = clampi((int)floorf((px - s.lox) / s.cell), 0, s.nx - 1);
  g.y = clampi((int)floorf((py - s.loy) / s.cell), 0, s.ny - 1);
  g.z = clampi((int)floorf((pz - s.loz) / s.cell), 0, s.nz - 1);
  return g;
}
__device__ __forceinline__ int cell_index(const SegParams &s, int3 g)
{
  return (g.z * s.ny + g.y) * s.nx + g.x;
}

// sph_common.glsl:84-91
__device__ __forceinline__ float w_poly6(float r2, float h2, float coef)
{
  if (r2 >= h2) return 0.0f;
  float d = h2 - r2;
  return coef * d * d * d;
}
// sph_common.glsl:111-118
__device__ __forceinline__ float w_spiky_grad(float r, float h, float coef)
{
  if (r >= h) return 0.0f;
  float d = h - r;
  return coef * d * d;
}
// sph_common.glsl:121-127
__device__ __forceinline__ float w_visc_lap(float r, float h, float coef)
{
  if (r >= h) return 0.0f;
  return coef * (h - r);
}

// Visit the candidate slots of the (2R+1)^3 cells around `base`, in the
// reference's order (dz, dy, dx, then slot), at most kMaxCellScan slots per
// cell (sph_lambda.glsl:39-56). Within one (dz, dy) row the x-adjacent cells
// are adjacent in grid order, so a row is one contiguous run unless one of its
// cells holds more than kMaxCellScan particles.
template <int R, class F>
__device__ __forceinline__ void for_each_candidate(const SegParams &s, const uint32_t *__restrict__ off,
                                                   int3 base, F &&f)
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
#pragma unroll 1
        for (uint32_t k = a; k < b; ++k) f((int)k);
      } else {
#pragma unroll 1
        for (int x = x0; x <= x1; ++x) {
          const uint32_t cs = __ldg(&off[row + x]);
          uint32_t ce = __ldg(&off[row + x + 1]);
          if (ce - cs > (uint32_t)kMaxCellScan) ce = cs + kMaxCellScan;
#pragma unroll 1
          for (uint32_t k = cs; k < ce; ++k) f((int)k);
        }
      }
    }
  }
}

__device__ __forceinline__ bool collider_occupied(const SegParams &s, const uint8_t *__restrict__ col, int cx,
                                                  int cy, int cz)
{
  if (cx < 0 || cy < 0 || cz < 0 || cx >= s.col_nx || cy >= s.col_ny || cz >= s.col_nz) return false;
  return col[s.col_begin + ((long long)cz * s.col_ny + cy) * s.col_nx + cx] != 0;
}
__device__ __forceinline__ int3 collider_coord(const SegParams &s, float px, float py, float pz)
{
  return make_int3((int)floorf((px - s.lox) / s.voxel), (int)floorf((py - s.loy) / s.voxel),
                   (int)floorf((pz - s.loz) / s.voxel));
}

// ---- launch wrappers (defined in the kernel translation units) ------------
// Block sizes are chosen per kernel by the tuner (runtime.cu); 0 = default.

// grid build
void launch_predict_key(const DeviceState &d, const float4 *normal_in, cudaStream_t st);
void launch_key_only(const DeviceState &d, const float4 *pred, cudaStream_t st);
void launch_scan(const DeviceState &d, cudaStream_t st);
// x_order: (predicted x, old slot) pairs from d.sort_x, the ids kept in
// d.rank_tmp for permute_step; else (id, old slot) pairs.
void launch_scatter(const DeviceState &d, cudaStream_t st, bool x_order = false);
void launch_cell_sort(const DeviceState &d, cudaStream_t st);
// FLOWX_FLAG_REFERENCE_ORDER in place of scatter + cell_sort: d.pairs from the
// reference's bitonic network over the keys predict_key / key_only left
// (the scan must have run); returns the number of kernels launched.
int launch_reference_order(const DeviceState &d, cudaStream_t st);
// writes pred_out and its copy in d.quads
void launch_permute_step(const DeviceState &d, float4 *pred_out, const float4 *normal_in, cudaStream_t st);
void launch_permute_all(const DeviceState &d, const float4 *pred_in, float4 *pred_out, cudaStream_t st);
// neighbour passes
void launch_normal(const DeviceState &d, const float4 *pred, float4 *out, cudaStream_t st);
void launch_lambda(const DeviceState &d, const float4 *pred, cudaStream_t st);
// d.quads <- pred (the per-pass API's lambda, whose input was not written
// by permute_step or delta_apply)
void launch_fill_quads(const DeviceState &d, const float4 *pred, cudaStream_t st);
// quad_bounds and row_yz from pred, for a lambda or XSPH pass over pred that
// trims its rows (d.trim)
void launch_row_bounds(const DeviceState &d, const float4 *pred, cudaStream_t st);
// fused substep (exact = the reference's expressions, else re-associated).
// lambda and xsph_finalize filter candidates from d.quads, which must hold
// `pred`: permute_step and delta_apply leave there what they write.
void launch_lambda_f(const DeviceState &d, const float4 *pred, bool exact, cudaStream_t st);
// last: the substep's final iteration, which also leaves d.xv for XSPH
void launch_delta_apply_f(const DeviceState &d, const float4 *pred_in, float4 *pred_out, bool exact, bool last,
                          cudaStream_t st);
// d.xv from pred and the substep's starting positions, for a substep with no
// Jacobi iteration
void launch_xsph_inputs(const DeviceState &d, const float4 *pred, bool exact, cudaStream_t st);
// normals: the XSPH pass also evaluates the next substep's normal pass (same
// positions, densities and grid) into d.normal_alt; the next substep then
// skips its normal pass, the caller vouching that nothing changed positions,
// densities, parameters, grid or slot order in between.
void launch_xsph_finalize_f(const DeviceState &d, const float4 *pred, float4 *pos_out, bool keep_delta, bool exact,
                            bool normals, cudaStream_t st);
void launch_normal_f(const DeviceState &d, const float4 *pred, float4 *out, bool exact, cudaStream_t st);
// The same passes one warp per particle (pbf_warp.cu), bit-identical to the
// thread-per-particle kernels; the launch_*_f wrappers call them when
// d.warp_passes is set.
void launch_lambda_w(const DeviceState &d, const float4 *pred, bool exact, cudaStream_t st);
void launch_delta_apply_w(const DeviceState &d, const float4 *pred_in, float4 *pred_out, bool exact, bool last,
                          cudaStream_t st);
void launch_xsph_finalize_w(const DeviceState &d, const float4 *pred, float4 *pos_out, bool keep_delta, bool exact,
                            bool normals, cudaStream_t st);
void launch_normal_w(const DeviceState &d, const float4 *pred, float4 *out, bool exact, cudaStream_t st);
// The splat of one segment (cells [cell_begin, cell_begin + cell_count)):
// refreshes those cells' position bounds, then gathers every sample.
void launch_splat_segment(const DeviceState &d, int seg, int cell_begin, int cell_count, const float *surface_lo,
                          float spacing, float kernel_radius, float mass, float rest, const int *dims, float *out,
                          cudaStream_t st);
// single reference passes (per-pass API)
void launch_predict(const DeviceState &d, float4 *pred, cudaStream_t st);
void launch_delta(const DeviceState &d, const float4 *pred, cudaStream_t st);
void launch_apply(const DeviceState &d, float4 *pred, cudaStream_t st);
void launch_velocity(const DeviceState &d, const float4 *pred, cudaStream_t st);
void launch_xsph(const DeviceState &d, const float4 *pred, cudaStream_t st);
void launch_finalize(const DeviceState &d, const float4 *pred, cudaStream_t st);
// layout conversion between caller id order and grid order
void launch_gather_by_id(const uint32_t *ids, const float4 *src_by_id, float4 *dst_by_slot, int n, cudaStream_t st);
void launch_scatter_by_id(const uint32_t *ids, const float4 *src_by_slot, float4 *dst_by_id, int n, cudaStream_t st);
void launch_reorder(const uint32_t *src_slot, const float4 *src, float4 *dst, int n, cudaStream_t st);
// analytic collider voxeliser
struct Primitive;
void launch_voxelize(uint8_t *grid, int nx, int ny, int nz, float ox, float oy, float oz, float voxel,
                     const void *prims, int nprims, cudaStream_t st);

}  // namespace flowx
