// Marching cubes on the GPU: the iso-surface extraction of
// solver/marching_cubes.py (extract, :191-280) over a float32 splat grid on
// the device, producing the same indexed mesh - same vertices, in the same
// order, with the same float64 coordinates, and the same triangles.
//
// The reference numbers a vertex the first time a triangle uses its lattice
// edge while it walks the cubes k, j, i (x fastest) and each cube's triangles
// in table order. Every cube touching a crossed lattice edge uses that edge,
// so its first user is the lowest-index cube touching it: for each of the
// two axes across the edge, the cube whose corner offset there is 1, or the
// cube at coordinate 0. Each cube therefore knows which of its edges it
// "owns", and the mesh comes from
//   classify   - per cube: the corner-sign case, its triangle count, the
//                number of crossed edges it owns;
//   scan       - exclusive prefix sums of both counts (vertex and triangle
//                bases, in cube order);
//   vertices   - each cube places its owned edges' vertices in the order its
//                triangles first use them, and records each one's index
//                under its lattice edge;
//   triangles  - each cube writes its triangles' vertex indices.
// Interpolation is float64 on the float32 samples, with the reference's
// expressions (the library is built without FMA contraction), so coordinates
// match bit for bit.
//
// The 256-case triangle table is derived at set-up the way the reference
// derives it (solver/marching_cubes.py:64-164): per-face contour segments
// paired by the corner signs (opening transition with the next closing one,
// faces wound counter-clockwise from outside), chained into loops, each loop
// fan-triangulated in reverse.
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "runtime.h"

namespace flowx {
namespace {

constexpr int kMaxTriangles = 5;  // per case (checked when the table is built)
constexpr int kMcBlock = 256;
constexpr int kMcTile = 2048;      // scan tile: 256 threads x 8 items

// solver/marching_cubes.py:25-63: corners, edges and faces in the
// conventional marching-cubes numbering the table is expressed in.
const int kCorners[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int kEdges[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int kFaces[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

struct McTables {
  int8_t tri[256][kMaxTriangles * 3];  // edge triples
  int8_t ntri[256];
  int8_t first[256][12];  // edges in the order the case's triangles first use them
  int8_t nfirst[256];
  uint16_t crossed[256];  // edges with a sign change
  int8_t walk[12][3];     // lower corner, upper corner, axis
  uint16_t owned[8];      // edges a cube owns, by (i == 0) | (j == 0) << 1 | (k == 0) << 2
};

int edge_of(int a, int b)
{
  for (int e = 0; e < 12; ++e)
    if ((kEdges[e][0] == a && kEdges[e][1] == b) || (kEdges[e][0] == b && kEdges[e][1] == a)) return e;
  return -1;
}

// The six faces wound counter-clockwise as seen from outside the cube
// (Newell normal against the face centre's outward direction).
void oriented_faces(int out[6][4])
{
  for (int f = 0; f < 6; ++f) {
    double nx = 0, ny = 0, nz = 0, cx = 0, cy = 0, cz = 0;
    for (int i = 0; i < 4; ++i) {
      const int *a = kCorners[kFaces[f][i]], *b = kCorners[kFaces[f][(i + 1) % 4]];
      nx += (double)(a[1] - b[1]) * (a[2] + b[2]);
      ny += (double)(a[2] - b[2]) * (a[0] + b[0]);
      nz += (double)(a[0] - b[0]) * (a[1] + b[1]);
      cx += a[0];
      cy += a[1];
      cz += a[2];
    }
    const double outward = nx * (cx / 4.0 - 0.5) + ny * (cy / 4.0 - 0.5) + nz * (cz / 4.0 - 0.5);
    for (int i = 0; i < 4; ++i) out[f][i] = outward > 0.0 ? kFaces[f][i] : kFaces[f][3 - i];
  }
}

bool build_tables(McTables &t, std::string &err)
{
  std::memset(&t, 0, sizeof(t));
  int faces[6][4];
  oriented_faces(faces);
  for (int c = 0; c < 256; ++c) {
    bool inside[8];
    for (int k = 0; k < 8; ++k) inside[k] = (c >> k) & 1;
    // successor edge of each opening edge, in insertion order
    std::vector<std::pair<int, int>> succ;
    for (int f = 0; f < 6; ++f) {
      std::vector<std::pair<bool, int>> trans;  // (opening, edge) walking the face
      for (int i = 0; i < 4; ++i) {
        const int a = faces[f][i], b = faces[f][(i + 1) % 4];
        if (inside[a] && !inside[b]) trans.push_back({true, edge_of(a, b)});
        else if (inside[b] && !inside[a]) trans.push_back({false, edge_of(a, b)});
      }
      const int count = (int)trans.size();
      for (int i = 0; i < count; ++i) {
        if (!trans[i].first) continue;
        for (int step = 1; step < count; ++step) {
          const auto &o = trans[(i + step) % count];
          if (!o.first) {
            bool found = false;
            for (auto &kv : succ)
              if (kv.first == trans[i].second) {
                kv.second = o.second;
                found = true;
              }
            if (!found) succ.push_back({trans[i].second, o.second});
            break;
          }
        }
      }
    }
    auto next_of = [&](int e) {
      for (auto &kv : succ)
        if (kv.first == e) return kv.second;
      return -1;
    };
    bool visited[12] = {};
    int ntri = 0;
    for (auto &kv : succ) {
      if (visited[kv.first]) continue;
      std::vector<int> loop;
      int e = kv.first;
      while (e >= 0 && !visited[e]) {
        visited[e] = true;
        loop.push_back(e);
        e = next_of(e);
      }
      if (e < 0) {
        err = "marching cubes table: open contour in case " + std::to_string(c);
        return false;
      }
      for (size_t i = 1; i + 1 < loop.size(); ++i) {
        if (ntri >= kMaxTriangles) {
          err = "marching cubes table: more than 5 triangles in case " + std::to_string(c);
          return false;
        }
        t.tri[c][3 * ntri + 0] = (int8_t)loop[0];
        t.tri[c][3 * ntri + 1] = (int8_t)loop[i + 1];
        t.tri[c][3 * ntri + 2] = (int8_t)loop[i];
        ++ntri;
      }
    }
    t.ntri[c] = (int8_t)ntri;
    uint16_t seen = 0;
    int nf = 0;
    for (int i = 0; i < 3 * ntri; ++i) {
      const int e = t.tri[c][i];
      if (!(seen & (1u << e))) {
        seen |= (uint16_t)(1u << e);
        t.first[c][nf++] = (int8_t)e;
      }
    }
    t.nfirst[c] = (int8_t)nf;
    uint16_t crossed = 0;
    for (int e = 0; e < 12; ++e)
      if (inside[kEdges[e][0]] != inside[kEdges[e][1]]) crossed |= (uint16_t)(1u << e);
    t.crossed[c] = crossed;
  }
  for (int e = 0; e < 12; ++e) {
    const int a = kEdges[e][0], b = kEdges[e][1];
    int axis = 0;
    for (int i = 0; i < 3; ++i)
      if (kCorners[a][i] != kCorners[b][i]) axis = i;
    const bool a_low = kCorners[a][axis] < kCorners[b][axis];
    t.walk[e][0] = (int8_t)(a_low ? a : b);
    t.walk[e][1] = (int8_t)(a_low ? b : a);
    t.walk[e][2] = (int8_t)axis;
  }
  // Owned edges: on each axis across the edge, the lower corner sits at
  // offset 1, or the cube is the first along that axis.
  for (int flags = 0; flags < 8; ++flags) {
    uint16_t m = 0;
    for (int e = 0; e < 12; ++e) {
      const int axis = t.walk[e][2];
      const int *d = kCorners[t.walk[e][0]];
      bool own = true;
      for (int b = 0; b < 3; ++b)
        if (b != axis && !(d[b] == 1 || ((flags >> b) & 1))) own = false;
      if (own) m |= (uint16_t)(1u << e);
    }
    t.owned[flags] = m;
  }
  return true;
}

const McTables *host_tables(std::string &err)
{
  static std::mutex mu;
  static McTables tables;
  static int state = 0;  // 0 unbuilt, 1 ok, -1 failed
  static std::string failure;
  std::lock_guard<std::mutex> lock(mu);
  if (state == 0) state = build_tables(tables, failure) ? 1 : -1;
  if (state < 0) {
    err = failure;
    return nullptr;
  }
  return &tables;
}

struct Lattice {
  int nx, ny, nz;
  double ox, oy, oz, spacing, iso;
};

__device__ __forceinline__ long long cube_count(const Lattice &L)
{
  return (long long)(L.nx - 1) * (L.ny - 1) * (L.nz - 1);
}

__device__ __forceinline__ void cube_coord(const Lattice &L, long long c, int &i, int &j, int &k)
{
  const long long cx = L.nx - 1, cy = L.ny - 1;
  i = (int)(c % cx);
  j = (int)((c / cx) % cy);
  k = (int)(c / (cx * cy));
}

__device__ __forceinline__ long long sample_index(const Lattice &L, int i, int j, int k)
{
  return ((long long)k * L.ny + j) * L.nx + i;
}

// Lattice edge of cube-local edge e: (lower corner sample) * 3 + axis.
__device__ __forceinline__ long long lattice_edge(const Lattice &L, const McTables &t, int i, int j, int k, int e)
{
  const int lo = t.walk[e][0];
  const int cx = (lo == 1 || lo == 2 || lo == 5 || lo == 6) ? 1 : 0;
  const int cy = (lo == 2 || lo == 3 || lo == 6 || lo == 7) ? 1 : 0;
  const int cz = lo >= 4 ? 1 : 0;
  return sample_index(L, i + cx, j + cy, k + cz) * 3 + t.walk[e][2];
}

// Also lists the cubes with triangles (the only ones with owned crossed edges
// or triangles to emit) for the vertex and triangle kernels, one atomic per
// warp; the list's order does not matter, every output position comes from
// the scans.
__global__ void __launch_bounds__(kMcBlock) k_mc_classify(const float *__restrict__ field, Lattice L,
                                                          const McTables *__restrict__ t,
                                                          uint8_t *__restrict__ cases, uint2 *__restrict__ counts,
                                                          uint32_t *__restrict__ active, uint32_t *__restrict__ nactive)
{
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = c < cube_count(L);
  int nt = 0;
  if (in) {
    int i, j, k;
    cube_coord(L, c, i, j, k);
    const long long base = sample_index(L, i, j, k);
    const long long nx = L.nx, nxy = (long long)L.nx * L.ny;
    const long long off[8] = {0, 1, 1 + nx, nx, nxy, 1 + nxy, 1 + nx + nxy, nx + nxy};
    int cs = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if ((double)__ldg(&field[base + off[q]]) >= L.iso) cs |= 1 << q;
    cases[c] = (uint8_t)cs;
    const int flags = (i == 0 ? 1 : 0) | (j == 0 ? 2 : 0) | (k == 0 ? 4 : 0);
    nt = t->ntri[cs];
    counts[c] = make_uint2((uint32_t)nt, (uint32_t)__popc((unsigned)(t->crossed[cs] & t->owned[flags])));
  }
  const unsigned ballot = __ballot_sync(0xffffffffu, nt > 0);
  if (ballot) {
    const int lane = threadIdx.x & 31, leader = __ffs((int)ballot) - 1;
    uint32_t slot = 0;
    if (lane == leader) slot = atomicAdd(nactive, (uint32_t)__popc(ballot));
    slot = __shfl_sync(0xffffffffu, slot, leader);
    if (nt > 0) active[slot + (uint32_t)__popc(ballot & ((1u << lane) - 1u))] = (uint32_t)c;
  }
}

// ---- exclusive scan of the (triangles, vertices) pairs ----------------------
__device__ __forceinline__ uint2 block_scan2(uint2 v, uint2 &total)
{
  __shared__ uint2 warp_sums[kMcBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint2 x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t a = __shfl_up_sync(0xffffffffu, x.x, o), b = __shfl_up_sync(0xffffffffu, x.y, o);
    if (lane >= o) {
      x.x += a;
      x.y += b;
    }
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint2 w = lane < kMcBlock / 32 ? warp_sums[lane] : make_uint2(0u, 0u);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t a = __shfl_up_sync(0xffffffffu, w.x, o), b = __shfl_up_sync(0xffffffffu, w.y, o);
      if (lane >= o) {
        w.x += a;
        w.y += b;
      }
    }
    if (lane < kMcBlock / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  total = warp_sums[kMcBlock / 32 - 1];
  const uint2 prefix = warp > 0 ? warp_sums[warp - 1] : make_uint2(0u, 0u);
  __syncthreads();
  return make_uint2(prefix.x + x.x - v.x, prefix.y + x.y - v.y);
}

__global__ void __launch_bounds__(kMcBlock) k_mc_tile_sums(const uint2 *__restrict__ in, long long n,
                                                           uint2 *__restrict__ sums)
{
  const long long base = (long long)blockIdx.x * kMcTile;
  uint2 local = make_uint2(0u, 0u);
  for (int q = 0; q < kMcTile / kMcBlock; ++q) {
    const long long idx = base + (long long)q * kMcBlock + threadIdx.x;
    if (idx < n) {
      const uint2 v = in[idx];
      local.x += v.x;
      local.y += v.y;
    }
  }
  uint2 total;
  block_scan2(local, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block: exclusive scan of the tile sums in place; the grand total last.
__global__ void __launch_bounds__(kMcBlock) k_mc_scan_sums(uint2 *__restrict__ sums, int nblocks,
                                                           uint2 *__restrict__ grand)
{
  uint2 carry = make_uint2(0u, 0u);
  for (int base = 0; base < nblocks; base += kMcBlock) {
    const int idx = base + threadIdx.x;
    const uint2 v = idx < nblocks ? sums[idx] : make_uint2(0u, 0u);
    uint2 total;
    const uint2 ex = block_scan2(v, total);
    if (idx < nblocks) sums[idx] = make_uint2(carry.x + ex.x, carry.y + ex.y);
    carry.x += total.x;
    carry.y += total.y;
  }
  if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(kMcBlock) k_mc_tile_scan(uint2 *__restrict__ io, long long n,
                                                           const uint2 *__restrict__ sums)
{
  const long long base = (long long)blockIdx.x * kMcTile + (long long)threadIdx.x * (kMcTile / kMcBlock);
  constexpr int kItems = kMcTile / kMcBlock;
  uint2 v[kItems];
  uint2 local = make_uint2(0u, 0u);
#pragma unroll
  for (int q = 0; q < kItems; ++q) {
    v[q] = base + q < n ? io[base + q] : make_uint2(0u, 0u);
    local.x += v[q].x;
    local.y += v[q].y;
  }
  uint2 total;
  uint2 run = block_scan2(local, total);
  const uint2 tile = sums[blockIdx.x];
  run.x += tile.x;
  run.y += tile.y;
#pragma unroll
  for (int q = 0; q < kItems; ++q) {
    if (base + q < n) io[base + q] = run;
    run.x += v[q].x;
    run.y += v[q].y;
  }
}

// solver/marching_cubes.py:258-276 for the edges a cube owns, in first-use
// order; one thread per listed cube.
__global__ void __launch_bounds__(kMcBlock) k_mc_vertices(const float *__restrict__ field, Lattice L,
                                                          const McTables *__restrict__ t,
                                                          const uint8_t *__restrict__ cases,
                                                          const uint2 *__restrict__ base_of,
                                                          const uint32_t *__restrict__ active, uint32_t nactive,
                                                          uint32_t *__restrict__ edge_vertex,
                                                          double *__restrict__ vertices)
{
  const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nactive) return;
  const long long c = active[a];
  const int cs = cases[c];
  if (cs == 0 || cs == 255) return;
  int i, j, k;
  cube_coord(L, c, i, j, k);
  const int flags = (i == 0 ? 1 : 0) | (j == 0 ? 2 : 0) | (k == 0 ? 4 : 0);
  const unsigned own = t->crossed[cs] & t->owned[flags];
  if (!own) return;
  const long long base = sample_index(L, i, j, k);
  const long long nx = L.nx, nxy = (long long)L.nx * L.ny;
  const long long off[8] = {0, 1, 1 + nx, nx, nxy, 1 + nxy, 1 + nx + nxy, nx + nxy};
  uint32_t idx = base_of[c].y;
  const int nf = t->nfirst[cs];
  for (int q = 0; q < nf; ++q) {
    const int e = t->first[cs][q];
    if (!(own & (1u << e))) continue;
    const int lo = t->walk[e][0], hi = t->walk[e][1], axis = t->walk[e][2];
    const double lo_value = (double)__ldg(&field[base + off[lo]]);
    const double hi_value = (double)__ldg(&field[base + off[hi]]);
    const double delta = hi_value - lo_value;
    const double tt = delta == 0.0 ? 0.5 : (L.iso - lo_value) / delta;
    const int dx = (lo == 1 || lo == 2 || lo == 5 || lo == 6) ? 1 : 0;
    const int dy = (lo == 2 || lo == 3 || lo == 6 || lo == 7) ? 1 : 0;
    const int dz = lo >= 4 ? 1 : 0;
    double p[3] = {L.ox + (double)(i + dx) * L.spacing, L.oy + (double)(j + dy) * L.spacing,
                   L.oz + (double)(k + dz) * L.spacing};
    p[axis] += tt * L.spacing;
    vertices[3 * (size_t)idx + 0] = p[0];
    vertices[3 * (size_t)idx + 1] = p[1];
    vertices[3 * (size_t)idx + 2] = p[2];
    edge_vertex[lattice_edge(L, *t, i, j, k, e)] = idx;
    ++idx;
  }
}

__global__ void __launch_bounds__(kMcBlock) k_mc_triangles(Lattice L, const McTables *__restrict__ t,
                                                           const uint8_t *__restrict__ cases,
                                                           const uint2 *__restrict__ base_of,
                                                           const uint32_t *__restrict__ active, uint32_t nactive,
                                                           const uint32_t *__restrict__ edge_vertex,
                                                           int32_t *__restrict__ triangles)
{
  const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nactive) return;
  const long long c = active[a];
  const int cs = cases[c];
  const int nt = t->ntri[cs];
  if (nt == 0) return;
  int i, j, k;
  cube_coord(L, c, i, j, k);
  const size_t out = 3 * (size_t)base_of[c].x;
  for (int q = 0; q < 3 * nt; ++q)
    triangles[out + q] = (int32_t)__ldg(&edge_vertex[lattice_edge(L, *t, i, j, k, t->tri[cs][q])]);
}

}  // namespace

// ---- host object ---------------------------------------------------------------
struct MarchingCubes {
  int device = 0;
  std::string err;
  McTables *d_tables = nullptr;
  uint8_t *cases = nullptr;
  uint2 *counts = nullptr, *tile_sums = nullptr, *grand = nullptr;
  uint32_t *edge_vertex = nullptr;
  uint32_t *active = nullptr, *nactive = nullptr;  // cubes with triangles, and how many
  double *vertices = nullptr;
  int32_t *triangles = nullptr;
  long long cap_cubes = 0, cap_counts = 0, cap_tiles = 0, cap_edges = 0, cap_vertices = 0, cap_triangles = 0;
  long long cap_active = 0;
  long long nvert = 0, ntri = 0;
  cudaStream_t last_stream = nullptr;

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
  int grow(T **p, long long &cap, long long need, const char *what)
  {
    if (need <= cap) return FLOWX_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = 0;
    int rc = cuda(cudaMalloc((void **)p, (size_t)std::max<long long>(need, 1) * sizeof(T)), what);
    if (!rc) cap = need;
    return rc;
  }
  void release()
  {
    void *ptrs[] = {d_tables, cases, counts, tile_sums, grand, edge_vertex, vertices, triangles, active, nactive};
    for (void *p : ptrs)
      if (p) cudaFree(p);
  }
};

}  // namespace flowx

using namespace flowx;

namespace {
thread_local std::string g_mc_create_error;
MarchingCubes *as_mc(flowx_mc *m) { return reinterpret_cast<MarchingCubes *>(m); }
}  // namespace

extern "C" {

int flowx_mc_case_table(int32_t mc_case, int32_t *edges, int32_t *triangle_count)
{
  if (mc_case < 0 || mc_case > 255 || !edges || !triangle_count) return FLOWX_ERR_ARG;
  std::string err;
  const McTables *t = host_tables(err);
  if (!t) return FLOWX_ERR_STATE;
  *triangle_count = t->ntri[mc_case];
  for (int q = 0; q < 3 * t->ntri[mc_case]; ++q) edges[q] = t->tri[mc_case][q];
  return FLOWX_OK;
}

int flowx_mc_create(int32_t device, flowx_mc **out)
{
  if (!out) {
    g_mc_create_error = "flowx_mc_create: out must not be NULL";
    return FLOWX_ERR_ARG;
  }
  *out = nullptr;
  std::string err;
  const McTables *t = host_tables(err);
  if (!t) {
    g_mc_create_error = err;
    return FLOWX_ERR_STATE;
  }
  MarchingCubes *m = new MarchingCubes();
  m->device = device;
  int rc = m->cuda(cudaSetDevice(device), "cudaSetDevice");
  if (!rc) rc = m->cuda(cudaMalloc((void **)&m->d_tables, sizeof(McTables)), "table allocation");
  if (!rc) rc = m->cuda(cudaMemcpy(m->d_tables, t, sizeof(McTables), cudaMemcpyHostToDevice), "table upload");
  if (!rc) rc = m->cuda(cudaMalloc((void **)&m->grand, sizeof(uint2)), "allocation");
  if (!rc) rc = m->cuda(cudaMalloc((void **)&m->nactive, sizeof(uint32_t)), "allocation");
  if (rc) {
    g_mc_create_error = m->err;
    m->release();
    delete m;
    return rc;
  }
  *out = reinterpret_cast<flowx_mc *>(m);
  return FLOWX_OK;
}

int flowx_mc_destroy(flowx_mc *mc)
{
  if (!mc) return FLOWX_OK;
  MarchingCubes *m = as_mc(mc);
  cudaSetDevice(m->device);
  // The last extraction ran on the caller's stream, which may already be
  // destroyed: cudaFree itself waits for the device's outstanding work.
  m->release();
  delete m;
  return FLOWX_OK;
}

const char *flowx_mc_last_error(const flowx_mc *mc)
{
  if (!mc) return g_mc_create_error.c_str();
  return reinterpret_cast<const MarchingCubes *>(mc)->err.c_str();
}

int flowx_mc_extract(flowx_mc *mc, const float *field, const int32_t dims[3], const double origin[3], double spacing,
                     double iso, void *stream, int64_t *vertex_count, int64_t *triangle_count)
{
  if (!mc) return FLOWX_ERR_ARG;
  MarchingCubes *m = as_mc(mc);
  cudaSetDevice(m->device);
  m->nvert = m->ntri = 0;
  if (!dims || !origin || !vertex_count || !triangle_count)
    return m->fail(FLOWX_ERR_ARG, "flowx_mc_extract: NULL argument");
  *vertex_count = *triangle_count = 0;
  if (dims[0] < 0 || dims[1] < 0 || dims[2] < 0) return m->fail(FLOWX_ERR_ARG, "negative lattice dims");
  if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2) return FLOWX_OK;  // no cube: empty mesh (marching_cubes.py:205)
  if (!field) return m->fail(FLOWX_ERR_ARG, "flowx_mc_extract: field is NULL");
  if (!(spacing > 0.0)) return m->fail(FLOWX_ERR_ARG, "spacing must be positive");
  const long long samples = (long long)dims[0] * dims[1] * dims[2];
  const long long cubes = (long long)(dims[0] - 1) * (dims[1] - 1) * (dims[2] - 1);
  if (samples * 3 > 0xffffffffll) return m->fail(FLOWX_ERR_CAPACITY, "lattice too large (3 x samples above 2^32)");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  m->last_stream = st;
  const long long tiles = (cubes + kMcTile - 1) / kMcTile;
  int rc = m->grow(&m->cases, m->cap_cubes, cubes, "case buffer");
  if (!rc) rc = m->grow(&m->counts, m->cap_counts, cubes, "count buffer");
  if (!rc) rc = m->grow(&m->tile_sums, m->cap_tiles, tiles, "scan buffer");
  if (!rc) rc = m->grow(&m->edge_vertex, m->cap_edges, samples * 3, "edge buffer");
  if (!rc) rc = m->grow(&m->active, m->cap_active, cubes, "active cube list");
  if (!rc) rc = m->cuda(cudaMemsetAsync(m->nactive, 0, sizeof(uint32_t), st), "active count reset");
  if (rc) return rc;
  Lattice L{dims[0], dims[1], dims[2], origin[0], origin[1], origin[2], spacing, iso};
  const unsigned nb = (unsigned)((cubes + kMcBlock - 1) / kMcBlock);
  k_mc_classify<<<nb, kMcBlock, 0, st>>>(field, L, m->d_tables, m->cases, m->counts, m->active, m->nactive);
  k_mc_tile_sums<<<(unsigned)tiles, kMcBlock, 0, st>>>(m->counts, cubes, m->tile_sums);
  k_mc_scan_sums<<<1, kMcBlock, 0, st>>>(m->tile_sums, (int)tiles, m->grand);
  k_mc_tile_scan<<<(unsigned)tiles, kMcBlock, 0, st>>>(m->counts, cubes, m->tile_sums);
  uint2 totals{0, 0};
  uint32_t nactive = 0;
  rc = m->cuda(cudaMemcpyAsync(&totals, m->grand, sizeof(uint2), cudaMemcpyDeviceToHost, st), "count read-back");
  if (!rc)
    rc = m->cuda(cudaMemcpyAsync(&nactive, m->nactive, sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
                 "count read-back");
  if (!rc) rc = m->cuda(cudaStreamSynchronize(st), "marching cubes count");
  if (rc) return rc;
  g_launches += 4;
  rc = m->grow(&m->vertices, m->cap_vertices, 3 * (long long)totals.y, "vertex buffer");
  if (!rc) rc = m->grow(&m->triangles, m->cap_triangles, 3 * (long long)totals.x, "triangle buffer");
  if (rc) return rc;
  const unsigned na = (unsigned)((nactive + kMcBlock - 1) / kMcBlock);
  if (totals.y > 0)
    k_mc_vertices<<<na, kMcBlock, 0, st>>>(field, L, m->d_tables, m->cases, m->counts, m->active, nactive,
                                           m->edge_vertex, m->vertices);
  if (totals.x > 0)
    k_mc_triangles<<<na, kMcBlock, 0, st>>>(L, m->d_tables, m->cases, m->counts, m->active, nactive, m->edge_vertex,
                                            m->triangles);
  g_launches += 2;
  rc = m->cuda(cudaGetLastError(), "flowx_mc_extract");
  if (rc) return rc;
  m->nvert = totals.y;
  m->ntri = totals.x;
  *vertex_count = totals.y;
  *triangle_count = totals.x;
  return FLOWX_OK;
}

int flowx_mc_download(flowx_mc *mc, double *vertices, size_t vertex_bytes, int32_t *triangles, size_t triangle_bytes)
{
  if (!mc) return FLOWX_ERR_ARG;
  MarchingCubes *m = as_mc(mc);
  cudaSetDevice(m->device);
  const size_t vb = (size_t)m->nvert * 3 * sizeof(double), tb = (size_t)m->ntri * 3 * sizeof(int32_t);
  if ((vb && (!vertices || vertex_bytes < vb)) || (tb && (!triangles || triangle_bytes < tb)))
    return m->fail(FLOWX_ERR_ARG, "mesh download buffers too small for the last extraction");
  cudaStream_t st = m->last_stream;
  int rc = FLOWX_OK;
  if (vb) rc = m->cuda(cudaMemcpyAsync(vertices, m->vertices, vb, cudaMemcpyDeviceToHost, st), "vertex download");
  if (!rc && tb)
    rc = m->cuda(cudaMemcpyAsync(triangles, m->triangles, tb, cudaMemcpyDeviceToHost, st), "triangle download");
  if (!rc) rc = m->cuda(cudaStreamSynchronize(st), "mesh download");
  return rc;
}

int flowx_mc_mesh(flowx_mc *mc, const double **vertices, const int32_t **triangles)
{
  if (!mc || !vertices || !triangles) return FLOWX_ERR_ARG;
  MarchingCubes *m = as_mc(mc);
  *vertices = m->vertices;
  *triangles = m->triangles;
  return FLOWX_OK;
}

}  // extern "C"
