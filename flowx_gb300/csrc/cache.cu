// Disk cache in the reference's FLWXCA01 format (solver/cache.py:12-34,
// :203-266, :339-421): per-frame (positions, velocities) snapshots at
// arithmetic offsets behind a header, written from and loaded into a
// context's device state.
//
// File layout (little-endian):
//   header: magic "FLWXCA01" (8 bytes), format_version u32 (2), flowx_version
//           (16 bytes, NUL padded), particle_count u32, seed_frame i32,
//           last_frame i32, fps f32, collider_count u32, then per collider a
//           u32 name length and the name bytes, then config_hash (32 bytes);
//   frames seed_frame + 1 .. last_frame, each positions (N x 4 f32) then
//           velocities (N x 4 f32), frame f at header_size + (f - seed_frame
//           - 1) * frame_size.
// last_frame is rewritten after every frame write, so a torn tail from a
// crash is ignored on load. The seed frame itself is never stored.
//
// Frames move between the file and the context through a pinned host
// buffer: a write downloads positions and velocities in particle-id order
// (flowx_download); a load installs them the way the reference's
// _apply_cached does (solver/sph.py:700-733): positions and velocities,
// predicted = positions, lambda zero, and a grid rebuilt from them.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "runtime.h"

namespace flowx {
namespace {

constexpr char kMagic[8] = {'F', 'L', 'W', 'X', 'C', 'A', '0', '1'};
constexpr uint32_t kFormatVersion = 2;
constexpr size_t kFixedHeader = 8 + 4 + 16 + 4 + 4 + 4 + 4 + 4;  // <8sI16sIiifI
constexpr size_t kHeaderReadBytes = 8192;                       // solver/cache.py:79

void put_u32(std::vector<uint8_t> &b, uint32_t v)
{
  for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
uint32_t get_u32(const uint8_t *p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }

}  // namespace

struct Cache {
  FILE *file = nullptr;
  std::string path, err;
  char flowx_version[16] = {};
  uint32_t particle_count = 0;
  int32_t seed_frame = 0, last_frame = 0;
  float fps = 0.0f;
  std::vector<std::string> colliders;
  uint8_t config_hash[32] = {};
  size_t header_size = 0;
  size_t frame_size = 0;
  float *pinned = nullptr;  // 2 x N x 4 floats (positions, velocities)
  size_t pinned_floats = 0;

  int fail(int code, const std::string &m)
  {
    err = m;
    return code;
  }

  std::vector<uint8_t> pack_header() const
  {
    std::vector<uint8_t> b(kMagic, kMagic + 8);
    put_u32(b, kFormatVersion);
    b.insert(b.end(), flowx_version, flowx_version + 16);
    put_u32(b, particle_count);
    put_u32(b, (uint32_t)seed_frame);
    put_u32(b, (uint32_t)last_frame);
    uint32_t fbits;
    std::memcpy(&fbits, &fps, 4);
    put_u32(b, fbits);
    put_u32(b, (uint32_t)colliders.size());
    for (const auto &name : colliders) {
      put_u32(b, (uint32_t)name.size());
      b.insert(b.end(), name.begin(), name.end());
    }
    b.insert(b.end(), config_hash, config_hash + 32);
    return b;
  }

  // Parse a header (solver/cache.py:224-266); false when the bytes are not ours.
  bool unpack_header(const uint8_t *d, size_t n)
  {
    if (n < kFixedHeader || std::memcmp(d, kMagic, 8) != 0 || get_u32(d + 8) != kFormatVersion) return false;
    std::memcpy(flowx_version, d + 12, 16);
    particle_count = get_u32(d + 28);
    seed_frame = (int32_t)get_u32(d + 32);
    last_frame = (int32_t)get_u32(d + 36);
    const uint32_t fbits = get_u32(d + 40);
    std::memcpy(&fps, &fbits, 4);
    const uint32_t count = get_u32(d + 44);
    size_t off = kFixedHeader;
    colliders.clear();
    for (uint32_t c = 0; c < count; ++c) {
      if (off + 4 > n) return false;
      const uint32_t len = get_u32(d + off);
      if (off + 4 + len > n) return false;
      colliders.emplace_back((const char *)d + off + 4, len);
      off += 4 + len;
    }
    if (off + 32 > n) return false;
    std::memcpy(config_hash, d + off, 32);
    header_size = off + 32;
    frame_size = (size_t)8 * 4 * particle_count;
    return true;
  }

  int write_header()
  {
    const std::vector<uint8_t> h = pack_header();
    if (std::fseek(file, 0, SEEK_SET) != 0 || std::fwrite(h.data(), 1, h.size(), file) != h.size() ||
        std::fflush(file) != 0)
      return fail(FLOWX_ERR_STATE, "writing the cache header failed: " + path);
    header_size = h.size();
    return FLOWX_OK;
  }

  int ensure_pinned()
  {
    const size_t need = (size_t)8 * particle_count;
    if (pinned && pinned_floats >= need) return FLOWX_OK;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    cudaError_t e = cudaMallocHost((void **)&pinned, std::max<size_t>(need, 1) * sizeof(float));
    if (e != cudaSuccess) return fail(FLOWX_ERR_CUDA, std::string("pinned cache buffer: ") + cudaGetErrorString(e));
    pinned_floats = need;
    return FLOWX_OK;
  }

  int check_frame(int32_t frame, bool for_read) const
  {
    if (frame <= seed_frame) return FLOWX_ERR_ARG;
    if (for_read && frame > last_frame) return FLOWX_ERR_ARG;
    return FLOWX_OK;
  }

  long long frame_offset(int32_t frame) const
  {
    return (long long)header_size + (long long)(frame - seed_frame - 1) * (long long)frame_size;
  }

  int write_frame_host(int32_t frame, const float *positions, const float *velocities)
  {
    if (check_frame(frame, false)) return FLOWX_OK;  // the seed frame is never stored (solver/cache.py:363)
    const size_t n4 = (size_t)4 * particle_count;
    if (std::fseek(file, frame_offset(frame), SEEK_SET) != 0 ||
        std::fwrite(positions, sizeof(float), n4, file) != n4 ||
        std::fwrite(velocities, sizeof(float), n4, file) != n4)
      return fail(FLOWX_ERR_STATE, "writing a cache frame failed: " + path);
    last_frame = std::max(last_frame, frame);
    return write_header();
  }

  int read_frame_host(int32_t frame, float *positions, float *velocities)
  {
    if (check_frame(frame, true)) return fail(FLOWX_ERR_ARG, "frame outside the cached range");
    const size_t n4 = (size_t)4 * particle_count;
    if (std::fseek(file, frame_offset(frame), SEEK_SET) != 0 ||
        std::fread(positions, sizeof(float), n4, file) != n4 || std::fread(velocities, sizeof(float), n4, file) != n4)
      return fail(FLOWX_ERR_STATE, "reading a cache frame failed: " + path);
    return FLOWX_OK;
  }

  void release()
  {
    if (file) std::fclose(file);
    file = nullptr;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
  }
};

}  // namespace flowx

using namespace flowx;

namespace {
thread_local std::string g_cache_open_error;
Cache *as_cache(flowx_cache *c) { return reinterpret_cast<Cache *>(c); }
}  // namespace

extern "C" {

int flowx_cache_create(const char *path, const flowx_cache_header *header, flowx_cache **out)
{
  if (!path || !header || !out || (header->collider_count > 0 && !header->collider_names)) {
    g_cache_open_error = "flowx_cache_create: NULL argument";
    return FLOWX_ERR_ARG;
  }
  *out = nullptr;
  if (header->particle_count < 0 || header->collider_count < 0) {
    g_cache_open_error = "flowx_cache_create: negative count";
    return FLOWX_ERR_ARG;
  }
  Cache *c = new Cache();
  c->path = path;
  std::memcpy(c->flowx_version, header->flowx_version, 16);
  c->particle_count = (uint32_t)header->particle_count;
  c->seed_frame = header->seed_frame;
  c->last_frame = header->seed_frame;
  c->fps = header->fps;
  for (int i = 0; i < header->collider_count; ++i)
    c->colliders.emplace_back(header->collider_names[i] ? header->collider_names[i] : "");
  std::memcpy(c->config_hash, header->config_hash, 32);
  c->frame_size = (size_t)8 * 4 * c->particle_count;
  c->file = std::fopen(path, "w+b");
  int rc = c->file ? c->write_header() : c->fail(FLOWX_ERR_STATE, std::string("cannot create ") + path);
  if (rc) {
    g_cache_open_error = c->err;
    c->release();
    delete c;
    return rc;
  }
  *out = reinterpret_cast<flowx_cache *>(c);
  return FLOWX_OK;
}

int flowx_cache_open(const char *path, flowx_cache **out)
{
  if (!path || !out) {
    g_cache_open_error = "flowx_cache_open: NULL argument";
    return FLOWX_ERR_ARG;
  }
  *out = nullptr;
  Cache *c = new Cache();
  c->path = path;
  c->file = std::fopen(path, "r+b");
  if (!c->file) {
    g_cache_open_error = std::string("cannot open ") + path;
    delete c;
    return FLOWX_ERR_STATE;
  }
  std::vector<uint8_t> head(kHeaderReadBytes);
  const size_t got = std::fread(head.data(), 1, head.size(), c->file);
  if (!c->unpack_header(head.data(), got)) {
    g_cache_open_error = std::string("not a FLWXCA01 version-2 cache: ") + path;
    c->release();
    delete c;
    return FLOWX_ERR_ARG;
  }
  *out = reinterpret_cast<flowx_cache *>(c);
  return FLOWX_OK;
}

int flowx_cache_close(flowx_cache *cache)
{
  if (!cache) return FLOWX_OK;
  Cache *c = as_cache(cache);
  c->release();
  delete c;
  return FLOWX_OK;
}

const char *flowx_cache_last_error(const flowx_cache *cache)
{
  if (!cache) return g_cache_open_error.c_str();
  return reinterpret_cast<const Cache *>(cache)->err.c_str();
}

int flowx_cache_info(const flowx_cache *cache, flowx_cache_header *header)
{
  if (!cache || !header) return FLOWX_ERR_ARG;
  const Cache *c = reinterpret_cast<const Cache *>(cache);
  std::memcpy(header->flowx_version, c->flowx_version, 16);
  header->particle_count = (int32_t)c->particle_count;
  header->seed_frame = c->seed_frame;
  header->last_frame = c->last_frame;
  header->fps = c->fps;
  header->collider_count = (int32_t)c->colliders.size();
  header->collider_names = nullptr;
  std::memcpy(header->config_hash, c->config_hash, 32);
  return FLOWX_OK;
}

const char *flowx_cache_collider_name(const flowx_cache *cache, int32_t index)
{
  if (!cache) return nullptr;
  const Cache *c = reinterpret_cast<const Cache *>(cache);
  if (index < 0 || index >= (int32_t)c->colliders.size()) return nullptr;
  return c->colliders[index].c_str();
}

int flowx_cache_write_frame_host(flowx_cache *cache, int32_t frame, const float *positions, const float *velocities)
{
  if (!cache) return FLOWX_ERR_ARG;
  Cache *c = as_cache(cache);
  if (c->particle_count && (!positions || !velocities)) return c->fail(FLOWX_ERR_ARG, "NULL frame buffers");
  return c->write_frame_host(frame, positions, velocities);
}

int flowx_cache_read_frame_host(flowx_cache *cache, int32_t frame, float *positions, float *velocities)
{
  if (!cache) return FLOWX_ERR_ARG;
  Cache *c = as_cache(cache);
  if (c->particle_count && (!positions || !velocities)) return c->fail(FLOWX_ERR_ARG, "NULL frame buffers");
  return c->read_frame_host(frame, positions, velocities);
}

int flowx_cache_write_frame(flowx_cache *cache, flowx_ctx *ctx, int32_t frame)
{
  if (!cache || !ctx) return FLOWX_ERR_ARG;
  Cache *c = as_cache(cache);
  Ctx *x = reinterpret_cast<Ctx *>(ctx);
  if ((uint32_t)x->total_particles != c->particle_count)
    return c->fail(FLOWX_ERR_ARG, "particle count changed - the cache file no longer matches the run");
  if (c->check_frame(frame, false)) return FLOWX_OK;  // the seed frame is never stored (solver/cache.py:363)
  int rc = c->ensure_pinned();
  if (rc) return rc;
  const size_t bytes = (size_t)16 * c->particle_count;
  float *pos = c->pinned, *vel = c->pinned + (size_t)4 * c->particle_count;
  rc = flowx_download(ctx, FLOWX_BUF_POSITIONS, pos, bytes);
  if (!rc) rc = flowx_download(ctx, FLOWX_BUF_VELOCITIES, vel, bytes);
  if (rc) return c->fail(rc, std::string("cache frame download: ") + x->err);
  return c->write_frame_host(frame, pos, vel);
}

int flowx_cache_load_frame(flowx_cache *cache, flowx_ctx *ctx, int32_t frame, const flowx_push *push)
{
  if (!cache || !ctx || !push) return FLOWX_ERR_ARG;
  Cache *c = as_cache(cache);
  Ctx *x = reinterpret_cast<Ctx *>(ctx);
  if ((uint32_t)x->total_particles != c->particle_count)
    return c->fail(FLOWX_ERR_ARG, "particle count differs from the cache file's");
  int rc = c->ensure_pinned();
  if (!rc) rc = c->read_frame_host(frame, c->pinned, c->pinned + (size_t)4 * c->particle_count);
  if (rc) return rc;
  const size_t bytes = (size_t)16 * c->particle_count;
  const float *pos = c->pinned, *vel = c->pinned + (size_t)4 * c->particle_count;
  // solver/sph.py:700-733: positions, velocities, predicted mirrors positions,
  // lambda zero, then the grid rebuilt from the predictions.
  std::vector<float> zeros((size_t)4 * c->particle_count, 0.0f);
  rc = flowx_upload(ctx, FLOWX_BUF_POSITIONS, pos, bytes);
  if (!rc) rc = flowx_upload(ctx, FLOWX_BUF_VELOCITIES, vel, bytes);
  if (!rc) rc = flowx_upload(ctx, FLOWX_BUF_PREDICTED, pos, bytes);
  if (!rc) rc = flowx_upload(ctx, FLOWX_BUF_LAMBDA, zeros.data(), bytes);
  if (!rc) rc = flowx_build_grid(ctx, push);
  if (rc) return c->fail(rc, std::string("cache frame load: ") + x->err);
  return FLOWX_OK;
}

}  // extern "C"
