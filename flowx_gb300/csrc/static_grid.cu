// flowx_build_grid_static: the neighbour-grid build into caller-owned device
// buffers, allocating nothing.
//
// Some callers cannot let a library allocate device memory: an application
// that reserves its whole device-memory budget at start-up and hands out
// pieces of it, or code running in a region where the implicit device-wide
// synchronisation of cudaMalloc / cudaFree is not allowed. For them this
// entry point takes the predicted positions and the output key and cell
// buffers as device pointers and keeps all of its own scratch (cell counters
// and offsets, ranks, sort pairs, the segment table) in one file-scope
// `static __device__` array sized for at most kStaticMaxParticles particles
// and kStaticMaxCells cells (about 5 MB, held by every GPU that loads the
// library until the process exits).
//
// Host code cannot take the array's device address directly, so it is
// fetched with cudaGetSymbolAddress once per device, during the first call
// made with that device current; make that first call before any stream
// capture. That first call is a warm-up: with lazy module loading it is
// where the runtime loads this module onto the device, which reserves the
// array and may synchronise the device. Calls after it allocate nothing.
// The cached address belongs to the device's primary context: after a
// cudaDeviceReset the library must not be used again in the process.
// All calls share the one array and it keeps the last call's contents: each
// call clears the cell counters, the only part that must start at zero, and
// calls whose GPU work overlaps race on it. So issue them on one stream and
// from one host thread at a time (each call enqueues several launches, and
// two threads' sequences on one stream can interleave).
#include <mutex>
#include <string>

#include "runtime.h"

namespace flowx {
namespace {

constexpr int kStaticMaxParticles = 65536;
constexpr int kStaticMaxCells = 262144;
constexpr int kStaticMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of each scratch array inside the static block.
constexpr size_t kOffCounts = 0;
constexpr size_t kOffOffsets = kOffCounts + align256(sizeof(uint32_t) * kStaticMaxCells);
constexpr size_t kOffBlockSums = kOffOffsets + align256(sizeof(uint32_t) * (kStaticMaxCells + 1));
constexpr size_t kOffBigCells = kOffBlockSums + align256(sizeof(uint32_t) * (kStaticMaxCells / 2048 + 2));
constexpr size_t kOffKeyTmp = kOffBigCells + align256(sizeof(uint32_t) * (kStaticMaxCells + 1));
constexpr size_t kOffRankTmp = kOffKeyTmp + align256(sizeof(uint32_t) * kStaticMaxParticles);
constexpr size_t kOffIds = kOffRankTmp + align256(sizeof(uint32_t) * kStaticMaxParticles);
constexpr size_t kOffPairs = kOffIds + align256(sizeof(uint32_t) * kStaticMaxParticles);
constexpr size_t kOffPairsTmp = kOffPairs + align256(sizeof(unsigned long long) * kStaticMaxParticles);
constexpr size_t kOffSegs = kOffPairsTmp + align256(sizeof(unsigned long long) * kStaticMaxParticles);
constexpr size_t kStaticBytes = kOffSegs + align256(sizeof(SegParams));

static __device__ __align__(256) unsigned char g_grid_scratch[kStaticBytes];

struct DeviceScratch {
  unsigned char *base = nullptr;
  int sm_count = 0;
};
std::mutex g_scratch_mu;
DeviceScratch g_scratch[kStaticMaxDevices];
thread_local std::string g_static_error;

int fail(int code, const std::string &msg)
{
  g_static_error = msg;
  return code;
}

// The segment constants go to the scratch by a kernel argument, not a copy
// from host memory.
__global__ void k_store_seg(SegParams *__restrict__ dst, SegParams s) { *dst = s; }

__global__ void k_iota(uint32_t *__restrict__ ids, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) ids[k] = (uint32_t)k;
}

// Keys in the reference layout (sph_grid_key.glsl:21-27 after the sort):
// (cell, particle id, 0, 0) per slot, padding slots (cell_count, slot).
__global__ void k_write_keys(const unsigned long long *__restrict__ pairs, const uint32_t *__restrict__ key_tmp,
                             int n, int key_count, int cells, float4 *__restrict__ keys)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= key_count) return;
  if (k < n) {
    const unsigned long long pr = pairs[k];
    const uint32_t slot = (uint32_t)pr;
    keys[k] = make_float4((float)key_tmp[slot], (float)(uint32_t)(pr >> 32), 0.0f, 0.0f);
  } else {
    keys[k] = make_float4((float)cells, (float)k, 0.0f, 0.0f);
  }
}

// Cell ranges in the reference layout (sph_cell_clear.glsl, sph_cell_range.glsl):
// [start, end) per cell, -1 for an empty cell.
__global__ void k_write_ranges(const uint32_t *__restrict__ off, int cells, float *__restrict__ start,
                               float *__restrict__ end)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cells) return;
  const uint32_t a = off[c], b = off[c + 1];
  start[c] = b > a ? (float)a : -1.0f;
  end[c] = b > a ? (float)b : -1.0f;
}

// Device address of the scratch block for the current device (set up on
// the first call made with that device current).
int scratch_for_current_device(DeviceScratch &out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(FLOWX_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kStaticMaxDevices) return fail(FLOWX_ERR_CAPACITY, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  DeviceScratch &s = g_scratch[dev];
  if (!s.base) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_grid_scratch);
    if (e != cudaSuccess)
      return fail(FLOWX_ERR_CUDA, std::string("cudaGetSymbolAddress of the grid scratch: ") + cudaGetErrorString(e));
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(FLOWX_ERR_CUDA, std::string("device attribute: ") + cudaGetErrorString(e));
    s.base = static_cast<unsigned char *>(ptr);
    s.sm_count = sms;
  }
  out = s;
  return FLOWX_OK;
}

}  // namespace
}  // namespace flowx

using namespace flowx;

extern "C" {

int flowx_build_grid_static(const float *predicted, int32_t particle_count, const flowx_push *push, float *keys,
                            int32_t key_count, float *cell_start, float *cell_end, void *stream)
{
  if (!push || (particle_count > 0 && !predicted) || !keys || !cell_start || !cell_end)
    return fail(FLOWX_ERR_ARG, "flowx_build_grid_static: NULL pointer argument");
  if (particle_count < 0 || key_count < particle_count)
    return fail(FLOWX_ERR_ARG, "flowx_build_grid_static: need 0 <= particle_count <= key_count");
  const long long cells = (long long)push->i_grid[0] * push->i_grid[1] * push->i_grid[2];
  if (push->i_grid[0] <= 0 || push->i_grid[1] <= 0 || push->i_grid[2] <= 0 || cells != push->i_grid[3] ||
      !(push->f_lo[3] > 0.0f))
    return fail(FLOWX_ERR_ARG, "flowx_build_grid_static: inconsistent grid in the push block");
  if (push->i_layout[0] != particle_count)
    return fail(FLOWX_ERR_ARG, "flowx_build_grid_static: push i_layout.x differs from particle_count");
  if (particle_count > kStaticMaxParticles)
    return fail(FLOWX_ERR_CAPACITY, "flowx_build_grid_static: " + std::to_string(particle_count) +
                                        " particles exceed the static scratch limit of " +
                                        std::to_string(kStaticMaxParticles));
  if (cells > kStaticMaxCells)
    return fail(FLOWX_ERR_CAPACITY, "flowx_build_grid_static: " + std::to_string(cells) +
                                        " cells exceed the static scratch limit of " + std::to_string(kStaticMaxCells));
  if ((reinterpret_cast<uintptr_t>(predicted) | reinterpret_cast<uintptr_t>(keys)) % 16 != 0)
    return fail(FLOWX_ERR_ARG, "flowx_build_grid_static: predicted and keys must be 16-byte aligned");
  DeviceScratch sc;
  int rc = scratch_for_current_device(sc);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char *b = sc.base;

  DeviceState d{};
  d.counts = reinterpret_cast<uint32_t *>(b + kOffCounts);
  d.offsets = reinterpret_cast<uint32_t *>(b + kOffOffsets);
  d.block_sums = reinterpret_cast<uint32_t *>(b + kOffBlockSums);
  d.big_cells = reinterpret_cast<uint32_t *>(b + kOffBigCells);
  d.key_tmp = reinterpret_cast<uint32_t *>(b + kOffKeyTmp);
  d.rank_tmp = reinterpret_cast<uint32_t *>(b + kOffRankTmp);
  d.ids = reinterpret_cast<uint32_t *>(b + kOffIds);
  d.pairs = reinterpret_cast<unsigned long long *>(b + kOffPairs);
  d.pairs_tmp = reinterpret_cast<unsigned long long *>(b + kOffPairsTmp);
  SegParams *segs = reinterpret_cast<SegParams *>(b + kOffSegs);
  d.segs = segs;
  d.nseg = 1;
  d.n = particle_count;
  d.cells = (int)cells;
  d.sm_count = sc.sm_count;

  SegParams s{};
  seg_from_push(*push, s);
  s.p_begin = 0;
  s.c_begin = 0;
  s.col_begin = 0;
  d.seg0 = s;
  d.cseg_base = -1;
  cudaError_t e = cudaMemsetAsync(d.counts, 0, sizeof(uint32_t) * (size_t)cells, st);
  if (e != cudaSuccess) return fail(FLOWX_ERR_CUDA, std::string("flowx_build_grid_static: ") + cudaGetErrorString(e));
  k_store_seg<<<1, 1, 0, st>>>(segs, s);
  long long launched = 1;
  if (particle_count > 0) {
    k_iota<<<(particle_count + 255) / 256, 256, 0, st>>>(d.ids, particle_count);
    launch_key_only(d, reinterpret_cast<const float4 *>(predicted), st);
    launched += 2;
  }
  launch_scan(d, st);
  launch_scatter(d, st);
  launch_cell_sort(d, st);
  // scan: 3 launches; scatter and the per-slot cell ranking: one each when
  // there are particles; the large-cell sorter: always one
  launched += 3 + (particle_count > 0 ? 2 : 0) + 1;
  if (key_count > 0) {
    k_write_keys<<<(key_count + 255) / 256, 256, 0, st>>>(d.pairs, d.key_tmp, particle_count, key_count, (int)cells,
                                                          reinterpret_cast<float4 *>(keys));
    launched += 1;
  }
  k_write_ranges<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(d.offsets, (int)cells, cell_start, cell_end);
  g_launches += launched + 1;
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FLOWX_ERR_CUDA, std::string("flowx_build_grid_static: ") + cudaGetErrorString(e));
  return FLOWX_OK;
}

const char *flowx_build_grid_static_error(void) { return g_static_error.c_str(); }

}  // extern "C"
