// Neighbour-grid build: the counting sort that replaces the reference's
// bitonic key sort (shaders/sph_grid_key.glsl, sph_sort.glsl,
// sph_cell_clear.glsl, sph_cell_range.glsl, driven by solver/sph.py:482-498).
//
//   1. predict_key  - per slot: the predicted position's cell key and its rank
//                     among the particles sharing that cell, from a
//                     warp-aggregated atomic on the cell's counter;
//   2. scan         - exclusive scan of the cell counters into cell offsets
//                     (three launches: tile sums, top-level scan, tile scan);
//                     counters are re-zeroed on the way, cells holding more
//                     than kSmallCellSort particles are listed;
//   3. scatter      - (id, old slot) to offset[key] + rank, in a scratch copy;
//   4. cell_sort    - order each cell by its pairs: every pair of a cell of
//                     at most kSmallCellSort particles counts the smaller pairs
//                     of its cell and moves to that rank (thread per slot), a
//                     block ranks each listed large cell; the result is the
//                     deterministic (cell, id) order;
//   5. permute      - move particle state into the new slot order.
//
// The sorted key column, the [start, end) of every cell and each cell's
// membership equal the reference's; within a cell the reference's bitonic
// network leaves an arbitrary order, this leaves ascending ids. The fused
// substep's build in the re-associated arithmetic (x_order) orders each cell
// by predicted x instead (ties by old slot): the slots of a stencil row then run
// in x, so the walk on coarse cells can trim a row to the particle's reach, and
// on cells of h a warp's lanes have more alike neighbourhoods.
#include "pbf_math.cuh"

namespace flowx {


static inline int blk(const DeviceState &d, KernelId k, int def) { return d.block[k] > 0 ? d.block[k] : def; }
static inline unsigned grid_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// ---- 1. predict + key + rank ---------------------------------------------
__device__ __forceinline__ void count_key(uint32_t *counts, uint32_t key, bool active, uint32_t &rank)
{
  const unsigned mask = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  const unsigned peers = __match_any_sync(mask, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&counts[key], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  rank = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// Order-preserving integer of a float (negative values reversed below the
// positive ones; NaN above +inf).
__device__ __forceinline__ uint32_t ordered_bits(float x)
{
  const uint32_t u = __float_as_uint(x);
  return u ^ ((u >> 31) ? 0xffffffffu : 0x80000000u);
}

// Fused substep: pos/vel/normal -> key, rank (the predicted position itself is
// recomputed by the permute, which is cheaper than storing and re-reading it;
// x_order keeps its x for the scatter).
template <int SEG>
__global__ void k_predict_key(DeviceState d, const float4 *__restrict__ normal_in)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = k < d.n;
  uint32_t key = 0;
  if (active) {
    const SegParams &s = slot_params<SEG>(d, k);
    const float4 p = d.pos[k];
    const float4 v = d.vel[k];
    const float4 n = s.sigma > 0.0f ? normal_in[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    float3 vo, q;
    predict_particle(s, p, v, n, vo, q);
    key = (uint32_t)(s.c_begin + cell_index(s, cell_coord(s, q.x, q.y, q.z)));
    d.key_tmp[k] = key;
    if (d.x_order) d.sort_x[k] = ordered_bits(q.x);
  }
  uint32_t rank = 0;
  count_key(d.counts, key, active, rank);
  if (active) d.rank_tmp[k] = rank;
}

// Key from an already-predicted position (flowx_build_grid after a separate
// predict, or a seed's zero-length build: solver/sph.py:606).
__global__ void k_key_only(DeviceState d, const float4 *__restrict__ pred)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = k < d.n;
  uint32_t key = 0;
  if (active) {
    const SegParams &s = d.segs[slot_segment(d, k)];
    const float4 q = pred[k];
    key = (uint32_t)(s.c_begin + cell_index(s, cell_coord(s, q.x, q.y, q.z)));
    d.key_tmp[k] = key;
  }
  uint32_t rank = 0;
  count_key(d.counts, key, active, rank);
  if (active) d.rank_tmp[k] = rank;
}

void launch_predict_key(const DeviceState &d, const float4 *normal_in, cudaStream_t st)
{
  if (d.n <= 0) return;
  with_seg_source(d, [&](auto tag) {
    constexpr int SEG = decltype(tag)::value;
    const int b = FLOWX_BLOCK(d, K_PREDICT_KEY, 256, (const void *)k_predict_key<SEG>);
    k_predict_key<SEG><<<grid_for(d.n, b), b, 0, st>>>(d, normal_in);
  });
}

cudaError_t const_segs_upload_grid(int base, const SegParams *s, int n, cudaStream_t st)
{
  return cudaMemcpyToSymbolAsync(c_segs, s, sizeof(SegParams) * n, sizeof(SegParams) * base, cudaMemcpyHostToDevice,
                                 st);
}

void launch_key_only(const DeviceState &d, const float4 *pred, cudaStream_t st)
{
  const int b = FLOWX_BLOCK(d, K_PREDICT_KEY, 256, k_key_only);
  if (d.n > 0) k_key_only<<<grid_for(d.n, b), b, 0, st>>>(d, pred);
}

// ---- 2. exclusive scan of the cell counters -----------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t &total)
{
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  total = warp_sums[kScanThreads / 32 - 1];
  const uint32_t warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0u;
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t *__restrict__ counts, int cells,
                                                              uint32_t *__restrict__ block_sums)
{
  const long long base = (long long)blockIdx.x * kScanTile;
  uint32_t local = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    long long c = base + (long long)j * kScanThreads + threadIdx.x;
    if (c < cells) local += counts[c];
  }
  uint32_t total;
  block_exclusive_scan(local, total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// One block: exclusive scan of the tile sums in place; offsets[cells] = total;
// resets the large-cell list.
__global__ void __launch_bounds__(kScanThreads) k_scan_top(uint32_t *__restrict__ block_sums, int nblocks,
                                                           uint32_t *__restrict__ offsets, int cells,
                                                           uint32_t *__restrict__ big_cells)
{
  uint32_t carry = 0;
  for (int base = 0; base < nblocks; base += kScanThreads) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < nblocks ? block_sums[i] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, total);
    if (i < nblocks) block_sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) {
    offsets[cells] = carry;
    big_cells[0] = 0;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(uint32_t *__restrict__ counts, int cells,
                                                            const uint32_t *__restrict__ block_sums,
                                                            uint32_t *__restrict__ offsets,
                                                            uint32_t *__restrict__ big_cells)
{
  // Each thread owns kScanItems consecutive cells of the tile.
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t local = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const long long c = base + j;
    v[j] = c < cells ? counts[c] : 0u;
    local += v[j];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(local, total) + block_sums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const long long c = base + j;
    if (c < cells) {
      offsets[c] = run;
      if (v[j] != 0u) counts[c] = 0u;
      if (v[j] > (uint32_t)kSmallCellSort) {
        const uint32_t slot = atomicAdd(&big_cells[0], 1u);
        big_cells[1 + slot] = (uint32_t)c;
      }
    }
    run += v[j];
  }
}

void launch_scan(const DeviceState &d, cudaStream_t st)
{
  const int cells = d.cells;
  const int nblocks = (int)grid_for(cells, kScanTile);
  k_scan_reduce<<<nblocks, kScanThreads, 0, st>>>(d.counts, cells, d.block_sums);
  k_scan_top<<<1, kScanThreads, 0, st>>>(d.block_sums, nblocks, d.offsets, cells, d.big_cells);
  k_scan_down<<<nblocks, kScanThreads, 0, st>>>(d.counts, cells, d.block_sums, d.offsets, d.big_cells);
}

// ---- 3. scatter ---------------------------------------------------------
// X_ORDER: the pair leads with the predicted x (d.sort_x) and the id waits in
// d.rank_tmp[k] (this thread's rank, just read) for permute_step.
template <bool X_ORDER>
__global__ void k_scatter(DeviceState d)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n) return;
  const uint32_t key = d.key_tmp[k];
  const uint32_t slot = d.offsets[key] + d.rank_tmp[k];
  const uint32_t id = d.ids[k];
  if (X_ORDER) {
    d.pairs_tmp[slot] = ((unsigned long long)d.sort_x[k] << 32) | (unsigned long long)(uint32_t)k;
    d.rank_tmp[k] = id;
  } else {
    d.pairs_tmp[slot] = ((unsigned long long)id << 32) | (unsigned long long)(uint32_t)k;
  }
}

void launch_scatter(const DeviceState &d, cudaStream_t st, bool x_order)
{
  const int b = FLOWX_BLOCK(d, K_SCATTER, 256, x_order ? (const void *)k_scatter<true> : (const void *)k_scatter<false>);
  if (d.n <= 0) return;
  if (x_order) k_scatter<true><<<grid_for(d.n, b), b, 0, st>>>(d);
  else k_scatter<false><<<grid_for(d.n, b), b, 0, st>>>(d);
}

// ---- 4. order each cell by its pairs ---------------------------------------
// Cells of at most kSmallCellSort particles: each slot's (id or x, old slot)
// pair counts the smaller pairs of its cell in the scatter's copy (old slots
// are unique, so the counts are a permutation of the cell's ranks) and moves
// there. A
// warp's slots mostly share one cell, whose pairs its loads then share.
__global__ void k_cell_rank(DeviceState d)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n) return;
  const unsigned long long pr = d.pairs_tmp[k];
  const uint32_t cell = __ldg(&d.key_tmp[(uint32_t)pr]);
  const uint32_t a = __ldg(&d.offsets[cell]);
  const uint32_t n = __ldg(&d.offsets[cell + 1]) - a;
  if (n > (uint32_t)kSmallCellSort) return;  // listed: k_cell_sort_large
  uint32_t rank = 0;
  for (uint32_t f = 0; f < n; ++f) rank += __ldg(&d.pairs_tmp[a + f]) < pr ? 1u : 0u;
  d.pairs[a + rank] = pr;
}

// Large cells (listed by the scan): a block ranks each element against all
// others of its cell, from the scatter's copy into place. O(n^2 / blockDim)
// per cell, so cells above kMaxRankSortCell keep the scatter's order.
__global__ void __launch_bounds__(256) k_cell_sort_large(DeviceState d)
{
  const uint32_t count = d.big_cells[0];
  for (uint32_t item = blockIdx.x; item < count; item += gridDim.x) {
    const uint32_t c = d.big_cells[1 + item];
    const uint32_t a = d.offsets[c], n = d.offsets[c + 1] - a;
    if (n > (uint32_t)kMaxRankSortCell) {  // uniform across the block
      for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) d.pairs[a + e] = d.pairs_tmp[a + e];
      continue;
    }
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
      const unsigned long long mine = d.pairs_tmp[a + e];
      uint32_t rank = 0;
      for (uint32_t f = 0; f < n; ++f) rank += d.pairs_tmp[a + f] < mine ? 1u : 0u;
      d.pairs[a + rank] = mine;
    }
  }
}

void launch_cell_sort(const DeviceState &d, cudaStream_t st)
{
  const int b = FLOWX_BLOCK(d, K_CELL_SORT_SMALL, 256, k_cell_rank);
  if (d.n > 0) k_cell_rank<<<grid_for(d.n, b), b, 0, st>>>(d);
  k_cell_sort_large<<<d.sm_count, 256, 0, st>>>(d);
}

// ---- 3'/4'. the reference's order (FLOWX_FLAG_REFERENCE_ORDER) -----------
// The reference orders its key array with a bitonic network: sph_grid_key.glsl
// writes entry i = (cell of particle id i, i) for i < n and (cell count, i)
// for the padding up to S = next power of two >= n, and solver/sph.py:488-495
// runs sph_sort.glsl for k = 2, 4, .., S and j = k/2, .., 1. Each step
// compare-exchanges the entries i and i ^ j (i with bit j clear), swapping
// when (key_i > key_partner) == ((i & k) == 0): by key only, so equal keys in
// a descending block swap too and the network is unstable, but it is a fixed
// function of the array. Running the same steps on the same array therefore
// leaves every particle where the reference's grid build leaves it; slot k
// then takes the particle of entry k. The pairs of one step are disjoint, so
// the order inside a step does not matter; steps with j < kBitonicTile of a
// k run on one tile in shared memory, the wider ones on global memory.
constexpr int kBitonicTile = 2048;

__device__ __forceinline__ void bitonic_cx(unsigned long long &x, unsigned long long &y, bool ascending)
{
  if (((x >> 32) > (y >> 32)) == ascending) {
    const unsigned long long t = x;
    x = y;
    y = t;
  }
}

// Entry id of the reference's key array from slot k's key (and the slot each
// id held before this build); the padding entries after it.
__global__ void k_bitonic_keys(DeviceState d)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.bitonic_n) return;
  if (t < d.n) {
    const uint32_t id = d.ids[t];
    d.bitonic[id] = ((unsigned long long)d.key_tmp[t] << 32) | id;
    d.bitonic_inv[id] = (uint32_t)t;
  } else {
    d.bitonic[t] = ((unsigned long long)(uint32_t)d.cells << 32) | (uint32_t)t;
  }
}

// One step (k, j), j >= kBitonicTile: thread t takes the t-th pair.
__global__ void k_bitonic_step(unsigned long long *__restrict__ a, int S, int k, int j)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S / 2) return;
  const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
  unsigned long long x = a[i], y = a[i | j];
  const unsigned long long x0 = x;
  bitonic_cx(x, y, (i & k) == 0);
  if (x != x0) {
    a[i] = x;
    a[i | j] = y;
  }
}

// Steps (k, j) for k = kmin, 2 kmin, .., kmax and j = min(k, tile) / 2, .., 1
// on one tile of `tile` entries per block (blockDim.x = tile / 2, one pair
// per thread and step).
__global__ void __launch_bounds__(kBitonicTile / 2) k_bitonic_local(unsigned long long *__restrict__ a, int tile,
                                                                    int kmin, int kmax)
{
  __shared__ unsigned long long sh[kBitonicTile];
  const int base = blockIdx.x * tile;
  for (int e = threadIdx.x; e < tile; e += blockDim.x) sh[e] = a[base + e];
  __syncthreads();
  const int t = threadIdx.x;
  for (int k = kmin; k <= kmax; k <<= 1) {
    for (int j = min(k, tile) >> 1; j > 0; j >>= 1) {
      const int li = ((t & ~(j - 1)) << 1) | (t & (j - 1));
      unsigned long long x = sh[li], y = sh[li | j];
      bitonic_cx(x, y, ((base + li) & k) == 0);
      sh[li] = x;
      sh[li | j] = y;
      __syncthreads();
    }
  }
  for (int e = threadIdx.x; e < tile; e += blockDim.x) a[base + e] = sh[e];
}

// New slot k takes the particle of entry k: (id << 32 | its old slot), as the
// scatter + cell sort leave d.pairs.
__global__ void k_bitonic_pairs(DeviceState d)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n) return;
  const uint32_t id = (uint32_t)d.bitonic[k];
  d.pairs[k] = ((unsigned long long)id << 32) | d.bitonic_inv[id];
}

int launch_reference_order(const DeviceState &d, cudaStream_t st)
{
  const int S = d.bitonic_n;
  int launched = 0;
  k_bitonic_keys<<<grid_for(S, 256), 256, 0, st>>>(d);
  ++launched;
  const int tile = S < kBitonicTile ? S : kBitonicTile;
  const int tiles = S / tile;
  k_bitonic_local<<<tiles, tile / 2, 0, st>>>(d.bitonic, tile, 2, tile);
  ++launched;
  for (int k = 2 * tile; k <= S; k <<= 1) {
    for (int j = k >> 1; j >= tile; j >>= 1) {
      k_bitonic_step<<<grid_for(S / 2, 256), 256, 0, st>>>(d.bitonic, S, k, j);
      ++launched;
    }
    k_bitonic_local<<<tiles, tile / 2, 0, st>>>(d.bitonic, tile, k, k);
    ++launched;
  }
  if (d.n > 0) {
    k_bitonic_pairs<<<grid_for(d.n, 256), 256, 0, st>>>(d);
    ++launched;
  }
  return launched;
}

// ---- 5. permute ---------------------------------------------------------
// Fused substep: new slot k takes old slot s. Positions are copied, the
// predicted position recomputed from (pos, vel, normal) exactly as predict did,
// the substep's normal (computed into scratch in the old order) moved to the
// new slot, and the slot's key and id recorded (x_order: the id the scatter
// left in rank_tmp). Velocity and lambda need no
// copy: the rest of the substep rewrites them before reading.
template <int SEG>
__global__ void k_permute_step(DeviceState d, float4 *__restrict__ pred_out, const float4 *__restrict__ normal_in)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n) return;
  const unsigned long long pr = d.pairs[k];
  const int s = (int)(uint32_t)pr;
  const SegParams &sp = slot_params<SEG>(d, k);
  const float4 p = d.pos[s];
  const float4 v = d.vel[s];
  const float4 n = sp.sigma > 0.0f ? normal_in[s] : make_float4(0.f, 0.f, 0.f, 0.f);
  float3 vo, q;
  predict_particle(sp, p, v, n, vo, q);
  if (sp.sigma > 0.0f) d.normal[k] = n;
  d.pos_alt[k] = p;
  pred_out[k] = make_float4(q.x, q.y, q.z, 1.0f);
  store_quad(d.quads, k, q.x, q.y, q.z);
  d.ids[k] = d.x_order ? d.rank_tmp[s] : (uint32_t)(pr >> 32);
  d.keys[k] = d.key_tmp[s];
}

void launch_permute_step(const DeviceState &d, float4 *pred_out, const float4 *normal_in, cudaStream_t st)
{
  if (d.n <= 0) return;
  with_seg_source(d, [&](auto tag) {
    constexpr int SEG = decltype(tag)::value;
    const int b = FLOWX_BLOCK(d, K_PERMUTE_STEP, 256, (const void *)k_permute_step<SEG>);
    k_permute_step<SEG><<<grid_for(d.n, b), b, 0, st>>>(d, pred_out, normal_in);
  });
}

// Standalone grid build: every per-particle array moves to its new slot
// (into the *_alt arrays; the caller copies them back).
__global__ void k_permute_all(DeviceState d, const float4 *__restrict__ pred_in, float4 *__restrict__ pred_out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n) return;
  const unsigned long long pr = d.pairs[k];
  const int s = (int)(uint32_t)pr;
  d.pos_alt[k] = d.pos[s];
  d.vel_alt[k] = d.vel[s];
  pred_out[k] = pred_in[s];
  d.normal_alt[k] = d.normal[s];
  d.delta_alt[k] = d.delta[s];
  d.lam_alt[k] = d.lam[s];
  d.ids[k] = (uint32_t)(pr >> 32);
  d.keys[k] = d.key_tmp[s];
}

void launch_permute_all(const DeviceState &d, const float4 *pred_in, float4 *pred_out, cudaStream_t st)
{
  const int b = FLOWX_BLOCK(d, K_PERMUTE_ALL, 256, k_permute_all);
  if (d.n > 0) k_permute_all<<<grid_for(d.n, b), b, 0, st>>>(d, pred_in, pred_out);
}

// ---- layout conversion --------------------------------------------------
__global__ void k_gather_by_id(const uint32_t *__restrict__ ids, const float4 *__restrict__ src,
                               float4 *__restrict__ dst, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = src[ids[k]];
}
__global__ void k_scatter_by_id(const uint32_t *__restrict__ ids, const float4 *__restrict__ src,
                                float4 *__restrict__ dst, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[ids[k]] = src[k];
}
__global__ void k_reorder(const uint32_t *__restrict__ src_slot, const float4 *__restrict__ src,
                          float4 *__restrict__ dst, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = src[src_slot[k]];
}

void launch_gather_by_id(const uint32_t *ids, const float4 *src, float4 *dst, int n, cudaStream_t st)
{
  if (n > 0) k_gather_by_id<<<grid_for(n, 256), 256, 0, st>>>(ids, src, dst, n);
}
void launch_scatter_by_id(const uint32_t *ids, const float4 *src, float4 *dst, int n, cudaStream_t st)
{
  if (n > 0) k_scatter_by_id<<<grid_for(n, 256), 256, 0, st>>>(ids, src, dst, n);
}
void launch_reorder(const uint32_t *src_slot, const float4 *src, float4 *dst, int n, cudaStream_t st)
{
  if (n > 0) k_reorder<<<grid_for(n, 256), 256, 0, st>>>(src_slot, src, dst, n);
}

}  // namespace flowx
