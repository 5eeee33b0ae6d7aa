// Collider voxeliser for triangle meshes (collision/__init__.py:304-367
// _rebuild_grid / _point_inside, union :225-242).
//
// The reference marks a voxel of the domain grid occupied when its centre lies
// inside a collider mesh: it casts a ray from the centre along world +z
// (M^-1 (0, 0, 1) in the mesh's local space, where Blender's BVH lives) and
// takes the parity of the hits, re-launching past each hit. Each mesh only
// marks voxels of the index range of its world bounding box (:259-262
// _index_range over domain/__init__.py:212-218 world_bounds: the box of the
// eight transformed corners of the local bounds). A mesh with a singular
// transform voxelises to nothing (:340-353).
//
// Here the same parity is counted exactly: world-space triangles in double
// precision, one warp per (x, y) column of the mesh's range. The vertical
// line through a column's centres crosses a triangle when the column point is
// inside the triangle's projection; the edge tests are watertight: an edge's
// function is evaluated from its lexicographically smaller endpoint, so the
// two triangles sharing it get exactly opposite values, and a point exactly on
// an edge or vertex is decided as the point displaced by (eps, eps^2) would be
// (simulation of simplicity), which lies in exactly one triangle of a planar
// fan. A crossing at height z flips the parity of every centre below z: the
// warp records one flip bit per crossing and counts them from the top.
// Triangles with no projected area cannot be crossed transversally and are
// skipped.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "runtime.h"

namespace flowx {
namespace {

struct Affine {  // rows of the world matrix's upper 3 x 4
  double m[12];
};

__global__ void k_mesh_world(const float *__restrict__ v, int n, Affine a, double *__restrict__ out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double x = v[3 * t], y = v[3 * t + 1], z = v[3 * t + 2];
#pragma unroll
  for (int r = 0; r < 3; ++r) out[3 * t + r] = ((a.m[4 * r] * x + a.m[4 * r + 1] * y) + a.m[4 * r + 2] * z) + a.m[4 * r + 3];
}

// orient(u, v, p) = (v - u) x (p - u), evaluated from the lexicographically
// smaller endpoint: edge_fn(u, v, p) == -edge_fn(v, u, p) exactly.
__device__ __forceinline__ double edge_fn(double ux, double uy, double vx, double vy, double px, double py)
{
  if (ux < vx || (ux == vx && uy < vy)) return (vx - ux) * (py - uy) - (vy - uy) * (px - ux);
  return -((ux - vx) * (py - vy) - (uy - vy) * (px - vx));
}

// Whether p is inside w.r.t. edge u -> v of a counterclockwise triangle, given
// e = edge_fn(u, v, p): strictly left, or on the edge and left of it once p is
// displaced by (eps, eps^2) (d/dpx of e is -(vy - uy), d/dpy is vx - ux).
__device__ __forceinline__ bool edge_in(double e, double ux, double uy, double vx, double vy)
{
  if (e != 0.0) return e > 0.0;
  const double dy = vy - uy;
  if (dy != 0.0) return dy < 0.0;
  return vx - ux > 0.0;
}

// Centres of voxels k in [k0, k1) strictly below z: how many.
__device__ __forceinline__ int centres_below(double z, double oz, double voxel, int k0, int k1)
{
  double t = (z - oz) / voxel - 0.5;
  int k;
  if (!(t > (double)k0)) {
    k = k0;
  } else if (!(t < (double)k1)) {
    k = k1;
  } else {
    k = (int)ceil(t);
  }
  while (k > k0 && oz + ((double)(k - 1) + 0.5) * voxel >= z) --k;
  while (k < k1 && oz + ((double)k + 0.5) * voxel < z) ++k;
  return k - k0;
}

// One warp per column: the lanes share the column's triangles, and each
// crossing toggles bit m (the number of centres below it) of the column's
// flip set in shared memory; the XOR of toggles commutes, so the result does
// not depend on which lane finds which crossing. Voxel r of the column is
// inside when the bits above r hold an odd count.
__global__ void k_mesh_columns(const double *__restrict__ w, const int32_t *__restrict__ tri, int ntri, int i0, int i1,
                               int j0, int j1, int k0, int k1, int nx, int ny, double ox, double oy, double oz,
                               double voxel, uint8_t *__restrict__ grid)
{
  extern __shared__ uint32_t column_flips[];
  const int ci = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // warp-uniform
  const int lane = threadIdx.x & 31;
  const int ncol_x = i1 - i0;
  const int ncol = ncol_x * (j1 - j0);
  if (ci >= ncol) return;
  const int i = i0 + ci % ncol_x, j = j0 + ci / ncol_x;
  const int nzr = k1 - k0;
  const int words = (nzr + 1 + 31) >> 5;
  uint32_t *f = column_flips + (threadIdx.x >> 5) * words;
  for (int q = lane; q < words; q += 32) f[q] = 0u;
  __syncwarp();
  const double px = ox + ((double)i + 0.5) * voxel;
  const double py = oy + ((double)j + 0.5) * voxel;
  for (int t = lane; t < ntri; t += 32) {
    const int ia = tri[3 * t], ib = tri[3 * t + 1], ic = tri[3 * t + 2];
    double ax = w[3 * ia], ay = w[3 * ia + 1], az = w[3 * ia + 2];
    double bx = w[3 * ib], by = w[3 * ib + 1], bz = w[3 * ib + 2];
    double cx = w[3 * ic], cy = w[3 * ic + 1], cz = w[3 * ic + 2];
    if (px < fmin(ax, fmin(bx, cx)) || px > fmax(ax, fmax(bx, cx)) || py < fmin(ay, fmin(by, cy)) ||
        py > fmax(ay, fmax(by, cy)))
      continue;
    const double area = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
    if (area == 0.0) continue;
    if (area < 0.0) {  // make the projection counterclockwise
      double s = bx; bx = cx; cx = s;
      s = by; by = cy; cy = s;
      s = bz; bz = cz; cz = s;
    }
    const double wa = edge_fn(bx, by, cx, cy, px, py);
    if (!edge_in(wa, bx, by, cx, cy)) continue;
    const double wb = edge_fn(cx, cy, ax, ay, px, py);
    if (!edge_in(wb, cx, cy, ax, ay)) continue;
    const double wc = edge_fn(ax, ay, bx, by, px, py);
    if (!edge_in(wc, ax, ay, bx, by)) continue;
    const double z = ((wa * az + wb * bz) + wc * cz) / ((wa + wb) + wc);
    const int m = centres_below(z, oz, voxel, k0, k1);
    atomicXor(&f[m >> 5], 1u << (m & 31));
  }
  __syncwarp();
  for (int r = lane; r < nzr; r += 32) {
    const int m0 = r + 1;  // crossings counted by voxel r: bits m0 .. nzr
    int q = m0 >> 5;
    uint32_t count = (uint32_t)__popc(f[q] & (0xffffffffu << (m0 & 31)));
    for (++q; q < words; ++q) count += (uint32_t)__popc(f[q]);
    if (count & 1u) grid[((size_t)(k0 + r) * ny + j) * nx + i] = 1;
  }
}

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

}  // namespace flowx

using namespace flowx;

extern "C" int flowx_voxelize_meshes(flowx_ctx *ctx, const flowx_mesh *meshes, int count, const int32_t dims[3],
                                     float voxel_size, const float origin[3])
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  if (count < 0 || (count > 0 && !meshes) || !dims || !origin || !(voxel_size > 0.0f))
    return c->fail(FLOWX_ERR_ARG, "bad voxelize_meshes arguments");
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return c->fail(FLOWX_ERR_ARG, "collider dims must be positive");
  const long long voxels = (long long)dims[0] * dims[1] * dims[2];
  if (voxels > c->cap_voxels) return c->fail(FLOWX_ERR_CAPACITY, "collider grid larger than max_collider_voxels");
  // every mesh's arguments are checked before anything is launched
  for (int q = 0; q < count; ++q) {
    const flowx_mesh &m = meshes[q];
    if (m.vertex_count < 0 || m.triangle_count < 0 || (m.vertex_count > 0 && !m.vertices) ||
        (m.triangle_count > 0 && !m.triangles))
      return c->fail(FLOWX_ERR_ARG, "mesh " + std::to_string(q) + ": bad vertex or triangle arrays");
    for (long long t = 0; t < 3LL * m.triangle_count; ++t)
      if (m.triangles[t] < 0 || m.triangles[t] >= m.vertex_count)
        return c->fail(FLOWX_ERR_ARG, "mesh " + std::to_string(q) + ": triangle index out of range");
  }
  int rc = c->cuda(cudaMemsetAsync(c->d.collider, 0, (size_t)voxels, c->stream), "collider clear");
  if (rc) return rc;
  const double vox = voxel_size, ox = origin[0], oy = origin[1], oz = origin[2];
  for (int q = 0; q < count; ++q) {
    const flowx_mesh &m = meshes[q];
    if (m.vertex_count == 0 || m.triangle_count == 0) continue;
    const float *M = m.matrix_world;
    Affine a;
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 4; ++k) a.m[4 * r + k] = M[4 * r + k];
    const double det = a.m[0] * (a.m[5] * a.m[10] - a.m[6] * a.m[9]) - a.m[1] * (a.m[4] * a.m[10] - a.m[6] * a.m[8]) +
                       a.m[2] * (a.m[4] * a.m[9] - a.m[5] * a.m[8]);
    if (det == 0.0) continue;  // singular transform: nothing, as the reference
    // world bounds: the eight transformed corners of the local bounds
    double llo[3] = {INFINITY, INFINITY, INFINITY}, lhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int v = 0; v < m.vertex_count; ++v)
      for (int r = 0; r < 3; ++r) {
        llo[r] = std::min(llo[r], (double)m.vertices[3 * v + r]);
        lhi[r] = std::max(lhi[r], (double)m.vertices[3 * v + r]);
      }
    double wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int corner = 0; corner < 8; ++corner) {
      const double x = corner & 1 ? lhi[0] : llo[0], y = corner & 2 ? lhi[1] : llo[1], z = corner & 4 ? lhi[2] : llo[2];
      for (int r = 0; r < 3; ++r) {
        const double wv = ((a.m[4 * r] * x + a.m[4 * r + 1] * y) + a.m[4 * r + 2] * z) + a.m[4 * r + 3];
        wlo[r] = std::min(wlo[r], wv);
        whi[r] = std::max(whi[r], wv);
      }
    }
    const double o3[3] = {ox, oy, oz};
    int lo3[3], hi3[3];
    for (int r = 0; r < 3; ++r) {
      lo3[r] = (int)std::max(0.0, std::floor((wlo[r] - o3[r]) / vox));
      hi3[r] = (int)std::min((double)dims[r], std::ceil((whi[r] - o3[r]) / vox));
    }
    if (lo3[0] >= hi3[0] || lo3[1] >= hi3[1] || lo3[2] >= hi3[2]) continue;
    const size_t ncol = (size_t)(hi3[0] - lo3[0]) * (hi3[1] - lo3[1]);
    const size_t b_v = align_up(sizeof(float) * 3 * (size_t)m.vertex_count);
    const size_t b_t = align_up(sizeof(int32_t) * 3 * (size_t)m.triangle_count);
    const size_t b_w = align_up(sizeof(double) * 3 * (size_t)m.vertex_count);
    const size_t need = b_v + b_t + b_w;
    if (need > c->mesh_cap) {
      rc = c->cuda(cudaStreamSynchronize(c->stream), "mesh scratch resize");
      if (rc) return rc;
      if (c->d_mesh) cudaFree(c->d_mesh);
      c->d_mesh = nullptr;
      c->mesh_cap = 0;
      rc = c->cuda(cudaMalloc(&c->d_mesh, need), "mesh scratch");
      if (rc) return rc;
      c->mesh_cap = need;
    }
    char *base = static_cast<char *>(c->d_mesh);
    float *d_v = reinterpret_cast<float *>(base);
    int32_t *d_t = reinterpret_cast<int32_t *>(base + b_v);
    double *d_w = reinterpret_cast<double *>(base + b_v + b_t);
    rc = c->cuda(cudaMemcpyAsync(d_v, m.vertices, sizeof(float) * 3 * (size_t)m.vertex_count, cudaMemcpyHostToDevice,
                                 c->stream),
                 "mesh vertex upload");
    if (!rc)
      rc = c->cuda(cudaMemcpyAsync(d_t, m.triangles, sizeof(int32_t) * 3 * (size_t)m.triangle_count,
                                   cudaMemcpyHostToDevice, c->stream),
                   "mesh triangle upload");
    if (rc) return rc;
    k_mesh_world<<<(m.vertex_count + 255) / 256, 256, 0, c->stream>>>(d_v, m.vertex_count, a, d_w);
    const int words = (hi3[2] - lo3[2] + 1 + 31) / 32;  // a column's flip bits, per warp
    k_mesh_columns<<<(unsigned)((ncol + 3) / 4), 128, (size_t)4 * words * sizeof(uint32_t), c->stream>>>(
        d_w, d_t, m.triangle_count, lo3[0], hi3[0], lo3[1], hi3[1], lo3[2], hi3[2], dims[0], dims[1], ox, oy, oz, vox,
        c->d.collider);
    g_launches += 2;
    // the next mesh's uploads reuse the scratch after these kernels (stream order)
  }
  c->collider_installed = true;
  std::memcpy(c->collider_dims, dims, sizeof(c->collider_dims));
  return c->check_launch("flowx_voxelize_meshes");
}

extern "C" int flowx_download_collider(flowx_ctx *ctx, uint8_t *host, size_t bytes)
{
  if (!ctx) return FLOWX_ERR_ARG;
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  cudaSetDevice(c->device);
  if (!c->collider_installed) return c->fail(FLOWX_ERR_STATE, "no collider grid installed");
  const size_t voxels = (size_t)c->collider_dims[0] * c->collider_dims[1] * c->collider_dims[2];
  if (!host || bytes != voxels)
    return c->fail(FLOWX_ERR_ARG, "collider download must be the grid's voxel count, " + std::to_string(voxels) +
                                      " bytes");
  int rc = c->cuda(cudaMemcpyAsync(host, c->d.collider, voxels, cudaMemcpyDeviceToHost, c->stream), "collider download");
  if (rc) return rc;
  return c->cuda(cudaStreamSynchronize(c->stream), "collider download");
}
