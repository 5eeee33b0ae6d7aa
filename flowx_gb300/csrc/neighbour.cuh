// Two-phase neighbour walk and the pass bodies of the fused substep.
//
// The reference scans the 27 cells around every particle in every neighbour
// pass (sph_lambda.glsl:39-70 and its siblings): ~216 candidates per particle
// at 8 particles per cell, of which ~15-20% lie within h. On a SIMT machine a
// per-candidate branch into the pair arithmetic costs the whole warp that
// arithmetic for nearly every candidate (some lane almost always accepts).
// So each pass walks its candidates twice, inside one thread:
//   phase 1 - for each of the nine (dz, dy) rows of the stencil (one
//             contiguous slot run, the three x-adjacent cells being adjacent
//             in grid order), set bit t of a 64-bit register mask when slot
//             a + t passes the pass's own distance test, evaluated with the
//             very expression the pass body uses;
//   phase 2 - run the pass body over the set bits, rows in order, slots
//             ascending.
// Phase 2 visits exactly the candidates the body would accept, in the
// reference's (row, slot) order, so the result equals a single scan's.
//
// Phase 1 runs over all nine rows first and leaves their masks in shared
// memory (nine 64-bit words per thread); phase 2 is then one loop over every
// set bit of every row, each lane moving to its next row when its current
// mask runs out. A warp so runs the body (busiest lane's accepted total)
// times instead of the sum over rows of the busiest lane's per-row count,
// which at 8-10 particles per cell is about 45 instead of 75.
//
// A particle with a row longer than 64 slots (dense regions, or a cell above
// the reference's MAX_CELL_SCAN) takes the per-row walk, which handles such
// rows by walking them directly.
#pragma once

#include "pbf_math.cuh"

namespace flowx {

constexpr int kRows = 9;

template <bool EXACT>
__device__ __forceinline__ float pair_r2(float dx, float dy, float dz)
{
  if (EXACT) return dx * dx + dy * dy + dz * dz;
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Visit the candidates k of the 3x3x3 stencil around `base` whose position
// pos[k] satisfies pair_r2<EXACT>(p - pos[k]) < lim2, in the reference's
// order; `f(k, within)` is called for each, within = true when the candidate
// passed that very test (so a body that tests r^2 < lim2 with the same
// expression may skip it). Rows whose run exceeds 64 slots are walked directly
// with the reference's per-cell MAX_CELL_SCAN cap, calling f(k, false) for
// every candidate of the row (the body then makes its own test).
template <bool EXACT, class F>
__device__ __forceinline__ void for_each_within_rows(const SegParams &s, const uint32_t *__restrict__ off,
                                                     const float4 *__restrict__ pos, float4 p, float lim2,
                                                     int3 base, F &&f)
{
  const int x0 = max(base.x - 1, 0), x1 = min(base.x + 1, s.nx - 1);
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const int z = base.z + (r / 3) - 1;
    const int y = base.y + (r % 3) - 1;
    if (z < 0 || z >= s.nz || y < 0 || y >= s.ny) continue;
    const int row = s.c_begin + (z * s.ny + y) * s.nx;
    const uint32_t ra = __ldg(&off[row + x0]);
    const uint32_t rb = __ldg(&off[row + x1 + 1]);
    if (rb - ra > 64u) {
#pragma unroll 1
      for (int x = x0; x <= x1; ++x) {
        const uint32_t cs = __ldg(&off[row + x]);
        uint32_t ce = __ldg(&off[row + x + 1]);
        if (ce - cs > (uint32_t)kMaxCellScan) ce = cs + kMaxCellScan;
#pragma unroll 1
        for (uint32_t k = cs; k < ce; ++k) f((int)k, false);
      }
      continue;
    }
    // phase 1: this row's candidates within reach, as bits
    unsigned long long mm = 0ull;
#pragma unroll 4
    for (uint32_t k = ra; k < rb; ++k) {
      const float4 q = __ldg(&pos[k]);
      const float r2 = pair_r2<EXACT>(p.x - q.x, p.y - q.y, p.z - q.z);
      if (r2 < lim2) mm |= 1ull << (k - ra);
    }
    // phase 2: the pass body over them, slots ascending
#pragma unroll 1
    while (mm) {
      const int t = __ffsll((long long)mm) - 1;
      mm &= mm - 1ull;
      f((int)ra + t, true);
    }
  }
}

// Dynamic shared memory a neighbour-pass launch of `block` threads needs:
// the row masks, nine per thread, laid out row-major across the block.
inline size_t row_mask_bytes(int block) { return (size_t)block * kRows * sizeof(unsigned long long); }

// Phase 1 of all nine rows into this thread's shared masks (mine[r * stride]).
// Returns false, leaving the masks incomplete, when a row is wider than 64
// slots (the particle then takes the per-row walk).
template <bool EXACT>
__device__ __forceinline__ bool build_row_masks(const SegParams &s, const uint32_t *__restrict__ off,
                                                const float4 *__restrict__ pos, float4 p, float lim2, int3 base,
                                                unsigned long long *mine, int stride)
{
  const int x0 = max(base.x - 1, 0), x1 = min(base.x + 1, s.nx - 1);
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const int z = base.z + (r / 3) - 1;
    const int y = base.y + (r % 3) - 1;
    unsigned long long mm = 0ull;
    if (z >= 0 && z < s.nz && y >= 0 && y < s.ny) {
      const int row = s.c_begin + (z * s.ny + y) * s.nx;
      const uint32_t ra = __ldg(&off[row + x0]);
      const uint32_t rb = __ldg(&off[row + x1 + 1]);
      if (rb - ra > 64u) return false;
      // four candidates per step: their accept bits packed into a nibble
      // and or-ed into the 32-bit half of the mask it falls in (offsets
      // are multiples of four, so a nibble never straddles the halves)
      uint32_t lo = 0u, hi = 0u;
      const uint32_t len = rb - ra;
#pragma unroll 1
      for (uint32_t o = 0; o < len; o += 4) {
        uint32_t nib = 0u;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const uint32_t k = ra + o + (uint32_t)u;
          if (o + (uint32_t)u < len) {
            const float4 q = __ldg(&pos[k]);
            const float r2 = pair_r2<EXACT>(p.x - q.x, p.y - q.y, p.z - q.z);
            nib |= (r2 < lim2 ? 1u : 0u) << u;
          }
        }
        if (o < 32u)
          lo |= nib << o;
        else
          hi |= nib << (o - 32u);
      }
      mm = ((unsigned long long)hi << 32) | lo;
    }
    mine[r * stride] = mm;
  }
  return true;
}

// pair_r2 of two candidates at once, from q - p: negating a difference is
// exact and squares drop the sign, so each lane equals pair_r2<EXACT>(p - q)
// bit for bit (EXACT: (dx*dx + dy*dy) + dz*dz, each operation rounded;
// FAST: the same fused multiply-adds as pair_r2).
template <bool EXACT>
__device__ __forceinline__ float2 pair_r2_x2(float2 qx, float2 qy, float2 qz, float2 npx, float2 npy, float2 npz)
{
  const float2 dx = __fadd2_rn(qx, npx), dy = __fadd2_rn(qy, npy), dz = __fadd2_rn(qz, npz);
  if (EXACT) return __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
  return __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
}

// Bounds of the current positions that let phase 1 skip candidates beyond
// reach (row_bounds in pbf.cu maintains them for the positions in the quads).
struct RowTrim {
  const float2 *__restrict__ quad_bounds;  // per quad: x-row prefix max of x at its last slot,
                                           // x-row suffix min of x at its first slot
  const float4 *__restrict__ row_yz;       // per cell: y, z bounds of its x-row neighbourhood
};

// Compare-exchange of the descending row-key sort: the larger key first.
__device__ __forceinline__ void row_key_exchange(uint32_t &a, uint32_t &b)
{
  const uint32_t hi = max(a, b);
  b = min(a, b);
  a = hi;
}

// The nine row keys sorted in descending order by a 25-comparator network.
__device__ __forceinline__ void sort_row_keys(uint32_t (&key)[kRows])
{
  row_key_exchange(key[0], key[1]);
  row_key_exchange(key[3], key[4]);
  row_key_exchange(key[6], key[7]);
  row_key_exchange(key[1], key[2]);
  row_key_exchange(key[4], key[5]);
  row_key_exchange(key[7], key[8]);
  row_key_exchange(key[0], key[1]);
  row_key_exchange(key[3], key[4]);
  row_key_exchange(key[6], key[7]);
  row_key_exchange(key[0], key[3]);
  row_key_exchange(key[3], key[6]);
  row_key_exchange(key[0], key[3]);
  row_key_exchange(key[1], key[4]);
  row_key_exchange(key[4], key[7]);
  row_key_exchange(key[1], key[4]);
  row_key_exchange(key[2], key[5]);
  row_key_exchange(key[5], key[8]);
  row_key_exchange(key[2], key[5]);
  row_key_exchange(key[1], key[3]);
  row_key_exchange(key[5], key[7]);
  row_key_exchange(key[2], key[6]);
  row_key_exchange(key[4], key[6]);
  row_key_exchange(key[2], key[4]);
  row_key_exchange(key[2], key[3]);
  row_key_exchange(key[5], key[6]);
}

// build_row_masks over the slot quads: the same masks, four candidates per
// three 16-byte loads. A row [ra, rb) is covered by the quads ra/4 .. (rb-1)/4;
// their accept bits are assembled in order, the ra % 4 bits of slots before
// ra shifted out and the bits from rb - ra on (slots past the row) cleared.
//
// Each lane tests its rows longest first. The masks do not depend on the
// order rows are tested in (each is stored at its own row), but a warp steps
// through each row as long as its busiest lane does: with the rows in stencil
// order the lanes' long rows fall on different steps (lanes in different
// cells, and particles whose current cell is not the one their slot is in),
// with them sorted the long rows run together. The rows' quad counts are read
// first (all eighteen bounds loads issued at once; each row's bounds wait in
// its mask slot), sorted as keys (count << 4 | row) by a 25-comparator
// network for nine inputs (each comparator a min and a max; it permutes the
// keys, so every row is still tested once), and the rows tested in that order.
template <bool EXACT>
__device__ __forceinline__ bool build_row_masks_quads(const SegParams &s, const uint32_t *__restrict__ off,
                                                      const SlotQuad *__restrict__ quads, float4 p, float lim2,
                                                      int3 base, unsigned long long *mine, int stride)
{
  const int x0 = max(base.x - 1, 0), x1 = min(base.x + 1, s.nx - 1);
  uint32_t key[kRows];
#pragma unroll
  for (int r = 0; r < kRows; ++r) {
    const int z = base.z + (r / 3) - 1;
    const int y = base.y + (r % 3) - 1;
    uint32_t ra = 0u, rb = 0u;
    if (z >= 0 && z < s.nz && y >= 0 && y < s.ny) {
      const int row = s.c_begin + (z * s.ny + y) * s.nx;
      ra = __ldg(&off[row + x0]);
      rb = __ldg(&off[row + x1 + 1]);
      if (rb - ra > 64u) return false;
    }
    const uint32_t nq = rb != ra ? ((rb + 3u) >> 2) - (ra >> 2) : 0u;
    key[r] = (nq << 4) | (uint32_t)r;
    mine[r * stride] = ((unsigned long long)rb << 32) | ra;  // the row's bounds until its mask replaces them
  }
  sort_row_keys(key);
  unsigned long long order = 0ull;  // the rows, longest first, four bits each
#pragma unroll
  for (int j = 0; j < kRows; ++j) order |= (unsigned long long)(key[j] & 15u) << (4 * j);
  const float2 npx = make_float2(-p.x, -p.x), npy = make_float2(-p.y, -p.y), npz = make_float2(-p.z, -p.z);
#pragma unroll 1
  for (int j = 0; j < kRows; ++j, order >>= 4) {
    const int r = (int)(order & 15ull);
    const unsigned long long bounds = mine[r * stride];
    const uint32_t ra = (uint32_t)bounds, rb = (uint32_t)(bounds >> 32);
    unsigned long long mm = 0ull;
    {
      const uint32_t len = rb - ra;
      if (len != 0u) {
        const uint32_t lead = ra & 3u;
        const uint32_t g0 = ra >> 2, g1 = (rb + 3u) >> 2;
        auto quad_bits = [&](uint32_t g) -> uint32_t {
          const float4 X = __ldg(&quads[g].x), Y = __ldg(&quads[g].y), Z = __ldg(&quads[g].z);
          const float2 a = pair_r2_x2<EXACT>(make_float2(X.x, X.y), make_float2(Y.x, Y.y), make_float2(Z.x, Z.y),
                                             npx, npy, npz);
          const float2 b = pair_r2_x2<EXACT>(make_float2(X.z, X.w), make_float2(Y.z, Y.w), make_float2(Z.z, Z.w),
                                             npx, npy, npz);
          return (a.x < lim2 ? 1u : 0u) | (a.y < lim2 ? 2u : 0u) | (b.x < lim2 ? 4u : 0u) | (b.y < lim2 ? 8u : 0u);
        };
        if (lead + len <= 64u) {
          // at most 16 quads: each enters a 64-bit window (hi:lo) from the
          // top, so after the last one quad t's bits sit at 64 - 4 (g1 - g0)
          // + 4 t, and slot ra + s at 64 - 4 (g1 - g0) + lead + s
          uint32_t lo = 0u, hi = 0u;
#pragma unroll 1
          for (uint32_t g = g0; g < g1; ++g) {
            const uint32_t nib = quad_bits(g);
            lo = __funnelshift_r(lo, hi, 4);
            hi = (hi >> 4) | (nib << 28);
          }
          mm = (((unsigned long long)hi << 32) | lo) >> (64u - 4u * (g1 - g0) + lead);
        } else {
          // 17 quads (a row of 62-64 slots starting off a quad boundary)
          uint32_t lo = 0u, hi = 0u, ex = 0u;
#pragma unroll 1
          for (uint32_t g = g0, sh = 0u; g < g1; ++g, sh += 4u) {
            const uint32_t nib = quad_bits(g);
            if (sh < 32u)
              lo |= nib << sh;
            else if (sh < 64u)
              hi |= nib << (sh - 32u);
            else
              ex = nib;
          }
          mm = (((unsigned long long)hi << 32) | lo) >> lead;
          mm |= (unsigned long long)ex << (64u - lead);
        }
        if (len < 64u) mm &= (1ull << len) - 1ull;
      }
    }
    mine[r * stride] = mm;
  }
  return true;
}

// Row masks one pass leaves for a later pass that tests the same positions
// against the same grid with the same reach (the lambda and delta passes of
// one Jacobi iteration): nine masks per slot, masks[r * n + slot], and a flag
// for particles that took the per-row walk.
struct MaskRecord {
  unsigned long long *masks;
  uint8_t *wide;
  int n;
  unsigned long long *chunk_masks;  // the trimmed walk's: its non-empty chunks, chunk_masks[j * n + slot]
  uint32_t *chunk_base;             // and the first slot of each
};


// The first t in [lo, hi) for which pred(t) is false, or hi, for a pred that
// is true on a prefix of the range and false after it (a binary search).
template <class P>
__device__ __forceinline__ uint32_t first_false(uint32_t lo, uint32_t hi, P &&pred)
{
#pragma unroll 1
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (pred(mid))
      lo = mid + 1u;
    else
      hi = mid;
  }
  return lo;
}

// The walk for cells coarser than the reach (rows of more than 64 slots):
// each stencil row's run trimmed to the particle's reach, then tested and
// visited sixteen quads at a time (a 64-bit mask in registers per chunk,
// its set bits visited at once), rows in order, slots ascending. The trim:
//   every candidate of the row lies within the y, z bounds of the row's
//   cells, so its squared distance is at least g^2, the squared y-z gap from
//   p to those bounds, and a row with g^2 beyond reach has no candidate;
//   otherwise a candidate can only be within reach when |x - p.x| < rx =
//   sqrt(reach^2 - g^2): the leading quads whose slots all lie left of
//   p.x - rx (the x-row's running maximum of x at their last slot says so)
//   and the trailing ones whose slots all lie right of p.x + rx (the running
//   minimum at their first slot) hold none. Both runs are monotone along the
//   row, so the first quad kept and the last are found by binary search.
// reach^2 is the test's lim2 widened by 2^-10 and the x window by 2^-20
// (|p.x| + rx), far above the rounding of the test and of these bounds, so
// every candidate the test accepts is visited, in the untrimmed walk's order.
// (A NaN coordinate of p makes every test reject, and its window comparisons
// fail, trimming nothing.) Slots in any order within a cell are handled; the
// x-ordered cells of the re-associated build make the trimmed runs short. A
// row above the reference's MAX_CELL_SCAN is walked cell by cell with the
// cap, as for_each_within_rows does.

// One stencil row of the trimmed walk: its run [ra, rb) and the quads
// [t0, t1) that can hold a candidate within reach (t0 == t1: none). False for
// a row above MAX_CELL_SCAN, which the caller walks cell by cell with the cap.
struct TrimmedRow {
  uint32_t ra, rb, t0, t1;
};

__device__ __forceinline__ bool trim_row(const SegParams &s, const uint32_t *__restrict__ off, RowTrim trim,
                                         float4 p, float reach2, int3 base, int x0, int x1, int r, TrimmedRow &t)
{
  t.ra = t.rb = t.t0 = t.t1 = 0u;
  const int z = base.z + (r / 3) - 1;
  const int y = base.y + (r % 3) - 1;
  if (z < 0 || z >= s.nz || y < 0 || y >= s.ny) return true;
  const int row = s.c_begin + (z * s.ny + y) * s.nx;
  const uint32_t ra = __ldg(&off[row + x0]);
  const uint32_t rb = __ldg(&off[row + x1 + 1]);
  t.ra = ra;
  t.rb = rb;
  if (rb <= ra) return true;
  if (rb - ra > (uint32_t)kMaxCellScan) return false;
  const float4 yz = __ldg(&trim.row_yz[row + base.x]);
  const float gy = fmaxf(fmaxf(yz.x - p.y, p.y - yz.y), 0.0f);
  const float gz = fmaxf(fmaxf(yz.z - p.z, p.z - yz.w), 0.0f);
  const float rx2 = reach2 - (gy * gy + gz * gz);
  if (!(rx2 > 0.0f)) return true;  // the whole row beyond reach
  uint32_t t0 = ra >> 2, t1 = (rb + 3u) >> 2;
  const float rx = sqrtf(rx2);
  const float tol = (fabsf(p.x) + rx) * 0x1p-20f;
  const float xlo = p.x - rx - tol, xhi = p.x + rx + tol;
  // leading quads whose last slot is in the row and whose running maximum
  // is left of the window; trailing quads whose first slot is in the row
  // and whose running minimum is right of it (both runs monotone in t)
  t0 = first_false(t0, min(t1, rb >> 2), [&](uint32_t q) { return __ldg(&trim.quad_bounds[q].x) < xlo; });
  const uint32_t lo_t = max(t0, (ra + 3u) >> 2);
  if (lo_t < t1)
    t1 = first_false(lo_t, t1, [&](uint32_t q) { return !(__ldg(&trim.quad_bounds[q].y) > xhi); });
  t.t0 = t0;
  t.t1 = t1;
  return true;
}

// The accept bits of the quads [c0, c1) (at most 16) of a row [ra, rb): each
// quad enters a 64-bit window (hi:lo) from the top, so after the last, slot
// 4 c0 + s sits at bit 64 - 4 (c1 - c0) + s; slots outside the row cleared.
template <bool EXACT>
__device__ __forceinline__ unsigned long long chunk_mask(const SlotQuad *__restrict__ quads, float2 npx, float2 npy,
                                                         float2 npz, float lim2, uint32_t c0, uint32_t c1,
                                                         uint32_t ra, uint32_t rb)
{
  uint32_t lo = 0u, hi = 0u;
#pragma unroll 1
  for (uint32_t g = c0; g < c1; ++g) {
    const float4 X = __ldg(&quads[g].x), Y = __ldg(&quads[g].y), Z = __ldg(&quads[g].z);
    const float2 a = pair_r2_x2<EXACT>(make_float2(X.x, X.y), make_float2(Y.x, Y.y), make_float2(Z.x, Z.y),
                                       npx, npy, npz);
    const float2 b = pair_r2_x2<EXACT>(make_float2(X.z, X.w), make_float2(Y.z, Y.w), make_float2(Z.z, Z.w),
                                       npx, npy, npz);
    const uint32_t nib =
        (a.x < lim2 ? 1u : 0u) | (a.y < lim2 ? 2u : 0u) | (b.x < lim2 ? 4u : 0u) | (b.y < lim2 ? 8u : 0u);
    lo = __funnelshift_r(lo, hi, 4);
    hi = (hi >> 4) | (nib << 28);
  }
  const uint32_t nq = c1 - c0;
  unsigned long long m = (((unsigned long long)hi << 32) | lo) >> (64u - 4u * nq);
  const uint32_t wb = 4u * c0;
  if (ra > wb) m &= ~((1ull << (ra - wb)) - 1ull);       // slots before the row
  if (rb - wb < 4u * nq) m &= (1ull << (rb - wb)) - 1ull;  // slots past it
  return m;
}

// The trimmed walk visiting as it tests: rows in order, each trimmed row's
// chunks tested and their set bits visited at once. REC: also records the
// non-empty chunks (mask and first slot) of slot i, up to kMaxChunks, for a
// later pass over the same positions (else, or with a row over
// MAX_CELL_SCAN, the slot is marked kChunksNotRecorded).
template <bool EXACT, bool REC = false, class F>
__device__ __forceinline__ void for_each_within_trimmed(const SegParams &s, const uint32_t *__restrict__ off,
                                                        const SlotQuad *__restrict__ quads, RowTrim trim, float4 p,
                                                        float lim2, int3 base, F &&f, MaskRecord rec = {}, int i = 0)
{
  uint32_t recorded = 0u;
  bool unrecorded = false;
  const int x0 = max(base.x - 1, 0), x1 = min(base.x + 1, s.nx - 1);
  const float2 npx = make_float2(-p.x, -p.x), npy = make_float2(-p.y, -p.y), npz = make_float2(-p.z, -p.z);
  const float reach2 = lim2 * (1.0f + 0x1p-10f);
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const int z = base.z + (r / 3) - 1;
    const int y = base.y + (r % 3) - 1;
    if (z < 0 || z >= s.nz || y < 0 || y >= s.ny) continue;
    const int row = s.c_begin + (z * s.ny + y) * s.nx;
    const uint32_t ra = __ldg(&off[row + x0]);
    const uint32_t rb = __ldg(&off[row + x1 + 1]);
    if (rb <= ra) continue;
    if (rb - ra > (uint32_t)kMaxCellScan) {
      unrecorded = true;
#pragma unroll 1
      for (int x = x0; x <= x1; ++x) {
        const uint32_t cs = __ldg(&off[row + x]);
        uint32_t ce = __ldg(&off[row + x + 1]);
        if (ce - cs > (uint32_t)kMaxCellScan) ce = cs + kMaxCellScan;
#pragma unroll 1
        for (uint32_t k = cs; k < ce; ++k) f((int)k, false);
      }
      continue;
    }
    const float4 yz = __ldg(&trim.row_yz[row + base.x]);
    const float gy = fmaxf(fmaxf(yz.x - p.y, p.y - yz.y), 0.0f);
    const float gz = fmaxf(fmaxf(yz.z - p.z, p.z - yz.w), 0.0f);
    const float rx2 = reach2 - (gy * gy + gz * gz);
    if (!(rx2 > 0.0f)) continue;  // the whole row beyond reach
    uint32_t t0 = ra >> 2, t1 = (rb + 3u) >> 2;
    const float rx = sqrtf(rx2);
    const float tol = (fabsf(p.x) + rx) * 0x1p-20f;
    const float xlo = p.x - rx - tol, xhi = p.x + rx + tol;
    t0 = first_false(t0, min(t1, rb >> 2), [&](uint32_t t) { return __ldg(&trim.quad_bounds[t].x) < xlo; });
    const uint32_t lo_t = max(t0, (ra + 3u) >> 2);
    if (lo_t < t1)
      t1 = first_false(lo_t, t1, [&](uint32_t t) { return !(__ldg(&trim.quad_bounds[t].y) > xhi); });
#pragma unroll 1
    for (uint32_t c0 = t0; c0 < t1; c0 += 16u) {
      const uint32_t c1 = min(c0 + 16u, t1), nq = c1 - c0;
      uint32_t lo = 0u, hi = 0u;
#pragma unroll 1
      for (uint32_t g = c0; g < c1; ++g) {
        const float4 X = __ldg(&quads[g].x), Y = __ldg(&quads[g].y), Z = __ldg(&quads[g].z);
        const float2 a = pair_r2_x2<EXACT>(make_float2(X.x, X.y), make_float2(Y.x, Y.y), make_float2(Z.x, Z.y),
                                           npx, npy, npz);
        const float2 b = pair_r2_x2<EXACT>(make_float2(X.z, X.w), make_float2(Y.z, Y.w), make_float2(Z.z, Z.w),
                                           npx, npy, npz);
        const uint32_t nib =
            (a.x < lim2 ? 1u : 0u) | (a.y < lim2 ? 2u : 0u) | (b.x < lim2 ? 4u : 0u) | (b.y < lim2 ? 8u : 0u);
        lo = __funnelshift_r(lo, hi, 4);
        hi = (hi >> 4) | (nib << 28);
      }
      unsigned long long m = (((unsigned long long)hi << 32) | lo) >> (64u - 4u * nq);
      const uint32_t wb = 4u * c0;
      if (ra > wb) m &= ~((1ull << (ra - wb)) - 1ull);       // slots before the row
      if (rb - wb < 4u * nq) m &= (1ull << (rb - wb)) - 1ull;  // slots past it
      if (REC && m != 0ull) {
        if (recorded < (uint32_t)kMaxChunks) {
          rec.chunk_masks[(size_t)recorded * rec.n + i] = m;
          rec.chunk_base[(size_t)recorded * rec.n + i] = wb;
          ++recorded;
        } else {
          unrecorded = true;
        }
      }
#pragma unroll 1
      while (m) {
        const int t = __ffsll((long long)m) - 1;
        m &= m - 1ull;
        f((int)(wb + (uint32_t)t), true);
      }
    }
  }
  if (REC) rec.wide[i] = unrecorded ? kChunksNotRecorded : (uint8_t)recorded;
}

// The trimmed walk of the lambda and XSPH passes: every row trimmed first
// (row order), then the rows' chunks tested, each lane's rows longest first,
// into staging slots in shared memory that keep the walk's order (a row's
// chunks follow those of the rows before it; the masks in the row-mask
// slots, their first slots after them: trimmed_walk_bytes), then the staged
// chunks visited in that order, flattened across chunks. A warp steps through
// each row as long as its busiest lane does, and the trimmed rows a lane can
// reach differ from lane to lane (about four of the nine on the reference's
// 2.25 h cells, 16-30 quads each); with them sorted the lanes' long rows run
// together. A particle with more than kRows chunks, or a row over
// MAX_CELL_SCAN, is walked again by the in-order walk (which records its
// chunks with REC).
// REC: the non-empty staged chunks (masks and first slots) are also recorded
// for slot i, in order, so that a later pass over the same positions can
// replay them (visit_recorded_chunks).
// Between the passes each row's entry of the first-slot area holds the row's
// staging slot (bits 24-31), its quad count (12-23) and its first quad
// kept, less the row's first quad (0-11): at most 129 quads each, since a
// row of more than MAX_CELL_SCAN slots sends the particle to the in-order
// walk.
template <bool EXACT, bool REC, class F>
__device__ __forceinline__ void for_each_within_trimmed_staged(const SegParams &s, const uint32_t *__restrict__ off,
                                                               const SlotQuad *__restrict__ quads, RowTrim trim,
                                                               float4 p, float lim2, int3 base, F &&f,
                                                               MaskRecord rec = {}, int i = 0)
{
  extern __shared__ unsigned long long row_masks[];
  unsigned long long *sm = row_masks + threadIdx.x;
  uint32_t *sb = reinterpret_cast<uint32_t *>(row_masks + kRows * blockDim.x) + threadIdx.x;
  const int stride = blockDim.x;
  const int x0 = max(base.x - 1, 0), x1 = min(base.x + 1, s.nx - 1);
  const float reach2 = lim2 * (1.0f + 0x1p-10f);
  uint32_t chunks = 0u;
  bool overflow = false;
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    TrimmedRow t;
    uint32_t info = 0u;
    if (!trim_row(s, off, trim, p, reach2, base, x0, x1, r, t)) {
      overflow = true;
    } else if (t.t1 > t.t0) {
      const uint32_t nq = t.t1 - t.t0;
      info = (min(chunks, 255u) << 24) | (nq << 12) | (t.t0 - (t.ra >> 2));
      chunks += (nq + 15u) >> 4;
    }
    sb[r * stride] = info;
  }
  if (overflow || chunks > (uint32_t)kRows) {
    for_each_within_trimmed<EXACT, REC>(s, off, quads, trim, p, lim2, base, f, rec, i);
    return;
  }
  uint32_t key[kRows];  // quad count << 4 | row
#pragma unroll
  for (int r = 0; r < kRows; ++r) key[r] = (((sb[r * stride] >> 12) & 0xfffu) << 4) | (uint32_t)r;
  sort_row_keys(key);
  unsigned long long order = 0ull;  // the rows, longest first, four bits each
#pragma unroll
  for (int j = 0; j < kRows; ++j) order |= (unsigned long long)(key[j] & 15u) << (4 * j);
  const float2 npx = make_float2(-p.x, -p.x), npy = make_float2(-p.y, -p.y), npz = make_float2(-p.z, -p.z);
#pragma unroll 1
  for (int j = 0; j < kRows; ++j, order >>= 4) {
    const int r = (int)(order & 15ull);
    const uint32_t info = sb[r * stride];
    const uint32_t nq = (info >> 12) & 0xfffu;
    if (nq == 0u) break;  // the rows after it hold nothing either
    const int row = s.c_begin + ((base.z + (r / 3) - 1) * s.ny + (base.y + (r % 3) - 1)) * s.nx;
    const uint32_t ra = __ldg(&off[row + x0]), rb = __ldg(&off[row + x1 + 1]);
    const uint32_t t0 = (ra >> 2) + (info & 0xfffu), t1 = t0 + nq;
    uint32_t slot = info >> 24;
#pragma unroll 1
    for (uint32_t c0 = t0; c0 < t1; c0 += 16u, ++slot) {
      const unsigned long long m = chunk_mask<EXACT>(quads, npx, npy, npz, lim2, c0, min(c0 + 16u, t1), ra, rb);
      sm[slot * stride] = m;
    }
  }
  // the staged chunks' first slots (every row's entry read first: a chunk's
  // staging slot may be a later row's entry)
  uint32_t info[kRows];
#pragma unroll
  for (int r = 0; r < kRows; ++r) info[r] = sb[r * stride];
#pragma unroll
  for (int r = 0; r < kRows; ++r) {
    const uint32_t nq = (info[r] >> 12) & 0xfffu;
    if (nq == 0u) continue;
    const int row = s.c_begin + ((base.z + (r / 3) - 1) * s.ny + (base.y + (r % 3) - 1)) * s.nx;
    uint32_t c0 = (__ldg(&off[row + x0]) >> 2) + (info[r] & 0xfffu);
    const uint32_t c1 = c0 + nq;
#pragma unroll 1
    for (uint32_t slot = info[r] >> 24; c0 < c1; c0 += 16u, ++slot) sb[slot * stride] = 4u * c0;
  }
  if (REC) {  // the non-empty chunks, in order
    uint32_t recorded = 0u;
#pragma unroll 1
    for (uint32_t k = 0; k < chunks; ++k) {
      const unsigned long long m = sm[k * stride];
      if (m == 0ull) continue;
      rec.chunk_masks[(size_t)recorded * rec.n + i] = m;
      rec.chunk_base[(size_t)recorded * rec.n + i] = sb[k * stride];
      ++recorded;
    }
    rec.wide[i] = (uint8_t)recorded;
  }
  uint32_t j = 0, wb = 0;
  unsigned long long m = 0ull;
#pragma unroll 1
  while (true) {
    while (m == 0ull && j < chunks) {
      m = sm[j * stride];
      wb = sb[j * stride];
      ++j;
    }
    if (m == 0ull) break;
    const int b = __ffsll((long long)m) - 1;
    m &= m - 1ull;
    f((int)(wb + (uint32_t)b), true);
  }
}

// Dynamic shared memory of a launch using the staged trimmed walk.
inline size_t trimmed_walk_bytes(int block)
{
  return (size_t)block * kRows * (sizeof(unsigned long long) + sizeof(uint32_t));
}

// Phase 2 from slot i's recorded chunks (for_each_within_trimmed_staged with REC,
// left by the launch just before on the same stream: same positions, grid
// and reach), flattened across chunks; a slot marked kChunksNotRecorded walks
// its trimmed rows again.
template <bool EXACT, class F>
__device__ __forceinline__ void visit_recorded_chunks(const SegParams &s, const uint32_t *__restrict__ off,
                                                      const SlotQuad *__restrict__ quads, RowTrim trim, float4 p,
                                                      float lim2, int3 base, MaskRecord rec, int i, F &&f)
{
  const uint8_t count = __ldg(&rec.wide[i]);
  if (count == kChunksNotRecorded) {
    for_each_within_trimmed<EXACT>(s, off, quads, trim, p, lim2, base, f);
    return;
  }
  uint32_t j = 0, wb = 0;
  unsigned long long m = 0ull;
#pragma unroll 1
  while (true) {
    if (m == 0ull) {  // (every recorded chunk holds a candidate)
      if (j >= count) break;
      m = __ldg(&rec.chunk_masks[(size_t)j * rec.n + i]);
      wb = __ldg(&rec.chunk_base[(size_t)j * rec.n + i]);
      ++j;
    }
    const int t = __ffsll((long long)m) - 1;
    m &= m - 1ull;
    f((int)(wb + (uint32_t)t), true);
  }
}

// Phase 2: every set bit of every row, rows in order, slots ascending; each
// lane moves to its next row when its current mask runs out. WORDS32: the
// current row's mask is taken as two 32-bit words (bits of slots ra + 0..31,
// then ra + 32..63), whose first set bit and clear are cheaper than the 64-bit
// ones; it pays where the body is short (delta_apply: 0.603 -> 0.593 ms on the
// 4M workload), not in lambda or XSPH (within 0.5%, slower).
template <bool WORDS32 = false, class F>
__device__ __forceinline__ void visit_row_masks(const SegParams &s, const uint32_t *__restrict__ off, int3 base,
                                                const unsigned long long *mine, int stride, F &&f)
{
  const int x0 = max(base.x - 1, 0);
  int r = -1;
  uint32_t ra = 0;
  if (WORDS32) {
    uint32_t lo = 0u, hi = 0u;
#pragma unroll 1
    while (true) {
      if (lo == 0u) {
        if (hi != 0u) {
          lo = hi;
          hi = 0u;
          ra += 32u;
        } else {
          unsigned long long m = 0ull;
          do {
            ++r;
          } while (r < kRows && (m = mine[r * stride]) == 0ull);
          if (r >= kRows) break;
          const int z = base.z + (r / 3) - 1;
          const int y = base.y + (r % 3) - 1;
          const int row = s.c_begin + (z * s.ny + y) * s.nx;
          ra = __ldg(&off[row + x0]);
          lo = (uint32_t)m;
          hi = (uint32_t)(m >> 32);
          if (lo == 0u) {
            lo = hi;
            hi = 0u;
            ra += 32u;
          }
        }
      }
      const int t = __ffs(lo) - 1;
      lo &= lo - 1u;
      f((int)ra + t, true);
    }
    return;
  }
  unsigned long long m = 0ull;
#pragma unroll 1
  while (true) {
    if (m == 0ull) {
      do {
        ++r;
      } while (r < kRows && (m = mine[r * stride]) == 0ull);
      if (r >= kRows) break;
      const int z = base.z + (r / 3) - 1;
      const int y = base.y + (r % 3) - 1;
      const int row = s.c_begin + (z * s.ny + y) * s.nx;
      ra = __ldg(&off[row + x0]);
    }
    const int t = __ffsll((long long)m) - 1;
    m &= m - 1ull;
    f((int)ra + t, true);
  }
}

// The two-phase walk with phase 2 flattened across rows (see the top of this
// file); launches must provide row_mask_bytes(blockDim.x) of dynamic shared
// memory. Same visits, same order as for_each_within_rows.
template <bool EXACT, class F>
__device__ __forceinline__ void for_each_within(const SegParams &s, const uint32_t *__restrict__ off,
                                                const float4 *__restrict__ pos, float4 p, float lim2, int3 base,
                                                F &&f)
{
  extern __shared__ unsigned long long row_masks[];
  unsigned long long *mine = row_masks + threadIdx.x;
  if (build_row_masks<EXACT>(s, off, pos, p, lim2, base, mine, blockDim.x))
    visit_row_masks(s, off, base, mine, blockDim.x, f);
  else
    for_each_within_rows<EXACT>(s, off, pos, p, lim2, base, f);
}

// for_each_within with phase 1 over the slot quads (quads[k / 4] lane k % 4
// holding pos[k]).
// TRIMMED: cells coarser than the reach, the trimmed walk (for_each_within_trimmed).
template <bool EXACT, bool TRIMMED, class F>
__device__ __forceinline__ void for_each_within(const SegParams &s, const uint32_t *__restrict__ off,
                                                const float4 *__restrict__ pos, const SlotQuad *__restrict__ quads,
                                                RowTrim trim, float4 p, float lim2, int3 base, F &&f)
{
  if (TRIMMED) {
    for_each_within_trimmed_staged<EXACT, false>(s, off, quads, trim, p, lim2, base, f);
    return;
  }
  extern __shared__ unsigned long long row_masks[];
  unsigned long long *mine = row_masks + threadIdx.x;
  if (build_row_masks_quads<EXACT>(s, off, quads, p, lim2, base, mine, blockDim.x))
    visit_row_masks(s, off, base, mine, blockDim.x, f);
  else
    for_each_within_rows<EXACT>(s, off, pos, p, lim2, base, f);
}

// for_each_within (phase 1 over the slot quads) that also records slot i's
// masks.
template <bool EXACT, bool TRIMMED, class F>
__device__ __forceinline__ void for_each_within_recording(const SegParams &s, const uint32_t *__restrict__ off,
                                                          const float4 *__restrict__ pos,
                                                          const SlotQuad *__restrict__ quads, RowTrim trim, float4 p,
                                                          float lim2, int3 base, MaskRecord rec, int i, F &&f)
{
  if (TRIMMED) {
    for_each_within_trimmed_staged<EXACT, true>(s, off, quads, trim, p, lim2, base, f, rec, i);
    return;
  }
  extern __shared__ unsigned long long row_masks[];
  unsigned long long *mine = row_masks + threadIdx.x;
  const int stride = blockDim.x;
  const bool ok = build_row_masks_quads<EXACT>(s, off, quads, p, lim2, base, mine, stride);
  rec.wide[i] = ok ? 0 : 1;
  if (ok) {
#pragma unroll
    for (int r = 0; r < kRows; ++r) rec.masks[(size_t)r * rec.n + i] = mine[r * stride];
    visit_row_masks(s, off, base, mine, stride, f);
  } else {
    for_each_within_rows<EXACT>(s, off, pos, p, lim2, base, f);
  }
}

// for_each_within from slot i's recorded masks, left by the launch just
// before on the same stream (same positions, grid and reach): phase 2 only.
// TRIMMED: the recording launch's chunks (visit_recorded_chunks).
template <bool EXACT, bool TRIMMED, class F>
__device__ __forceinline__ void for_each_within_recorded(const SegParams &s, const uint32_t *__restrict__ off,
                                                         const float4 *__restrict__ pos,
                                                         const SlotQuad *__restrict__ quads, RowTrim trim, float4 p,
                                                         float lim2, int3 base, MaskRecord rec, int i, F &&f)
{
  if (TRIMMED) {
    visit_recorded_chunks<EXACT>(s, off, quads, trim, p, lim2, base, rec, i, f);
    return;
  }
  extern __shared__ unsigned long long row_masks[];
  unsigned long long *mine = row_masks + threadIdx.x;
  const int stride = blockDim.x;
  if (__ldg(&rec.wide[i])) {
    for_each_within_rows<EXACT>(s, off, pos, p, lim2, base, f);
    return;
  }
#pragma unroll
  for (int r = 0; r < kRows; ++r) mine[r * stride] = __ldg(&rec.masks[(size_t)r * rec.n + i]);
  visit_row_masks<true>(s, off, base, mine, stride, f);
}

// sph_velocity.glsl:20-23 for one slot.
__device__ __forceinline__ float3 slot_velocity(const float4 &q, const float4 &p, float dtc)
{
  return make_float3((q.x - p.x) / dtc, (q.y - p.y) / dtc, (q.z - p.z) / dtc);
}

// What the XSPH pass needs of slot i besides its position: the velocity
// sph_velocity.glsl:20-23 derives from pred and the substep's starting
// position (the same expression XSPH evaluated per neighbour), and the
// density floor sph_xsph.glsl applies.
template <bool EXACT>
__device__ __forceinline__ float4 xsph_input(const SegParams &s, const DeviceState &d, int i, float4 q)
{
  const float4 p0 = d.pos_alt[i];
  const float dtc = s.dtc;
  float3 v;
  if (EXACT) {
    v = slot_velocity(q, p0, dtc);
  } else {
    const float inv_dtc = 1.0f / dtc;
    v = make_float3(__fmul_rn(__fsub_rn(q.x, p0.x), inv_dtc), __fmul_rn(__fsub_rn(q.y, p0.y), inv_dtc),
                    __fmul_rn(__fsub_rn(q.z, p0.z), inv_dtc));
  }
  return make_float4(v.x, v.y, v.z, fmaxf(d.lam[i].x, 1e-6f));
}

// ---- pass bodies ----------------------------------------------------------
// EXACT: the reference's expressions, operation for operation (bit-identical
// to the oracle). FAST: the same quantities re-associated for throughput (FMA,
// one reciprocal square root per pair, reciprocal-multiplies for divisions by
// per-particle constants), within float32 rounding of EXACT.

template <bool EXACT>
struct LambdaAcc {
  float density = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f, gn2 = 0.0f;

  // Pairs with r2 >= h2 contribute nothing (sph_lambda.glsl:58-62), so the
  // walk may skip them. The particle itself (r2 exactly 0) adds its density
  // and no gradient, which the r2 <= 1e-12 test gives without a test of j == i.
  __device__ __forceinline__ void pair(const SegParams &s, float dx, float dy, float dz, bool within)
  {
    if (EXACT) {
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (!within && r2 >= s.h2) return;
      density += s.mass * w_poly6(r2, s.h2, s.poly6);
      if (r2 <= 1e-12f) return;
      const float r = sqrtf(r2);
      const float sg = s.mass * w_spiky_grad(r, s.h, s.spiky);
      const float ax = sg * (dx / r), ay = sg * (dy / r), az = sg * (dz / r);
      gx += ax;
      gy += ay;
      gz += az;
      gn2 += ax * ax + ay * ay + az * az;
    } else {
      const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
      if (!within && r2 >= s.h2) return;
      const float t = __fsub_rn(s.h2, r2);
      density = __fmaf_rn(__fmul_rn(t, t), t, density);  // scaled by mass * poly6 at the end
      if (r2 <= 1e-12f) return;
      const float rinv = rsqrtf(r2);
      const float hr = __fsub_rn(s.h, __fmul_rn(r2, rinv));
      const float g = __fmul_rn(__fmul_rn(s.mass_spiky, __fmul_rn(hr, hr)), rinv);
      gx = __fmaf_rn(g, dx, gx);
      gy = __fmaf_rn(g, dy, gy);
      gz = __fmaf_rn(g, dz, gz);
      gn2 = __fmaf_rn(__fmul_rn(g, g), r2, gn2);
    }
  }

  __device__ __forceinline__ float2 finish(const SegParams &s) const
  {
    const float rest = s.rest;
    const float dens = EXACT ? density : __fmul_rn(density, s.mass * s.poly6);
    const float constraint = fmaxf(dens, 1e-6f) / rest - 1.0f;
    const float denom = (gx * gx + gy * gy + gz * gz + gn2) / (rest * rest) + s.eps;
    return make_float2(fmaxf(dens, 1e-6f), -constraint / fmaxf(denom, 1e-9f));
  }
};

template <bool EXACT>
__device__ __forceinline__ void delta_pair(const SegParams &s, float lambda_i, float lambda_j, float dx, float dy,
                                           float dz, float r2, float &ax, float &ay, float &az)
{
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
    ax += sc * (dx / r);
    ay += sc * (dy / r);
    az += sc * (dz / r);
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
    const float sc = __fmul_rn(__fmul_rn(lam, __fmul_rn(s.spiky, __fmul_rn(hr, hr))), rinv);
    ax = __fmaf_rn(sc, dx, ax);
    ay = __fmaf_rn(sc, dy, ay);
    az = __fmaf_rn(sc, dz, az);
  }
}

}  // namespace flowx
