// Host-side context of libflowx (private to the library).
#pragma once

#include <atomic>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/flowx.h"
#include "flowx_internal.cuh"

namespace flowx {

extern std::atomic<long long> g_launches;
float bits_to_float(int32_t b);
void seg_from_push(const flowx_push &p, SegParams &s);

// (iterations, substeps, starting predicted buffer, cells, normal pass on, flags,
// first substep's normal pass already evaluated by the previous XSPH pass)
using GraphKey = std::tuple<int, int, int, int, int, int, int>;
struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
};

struct Ctx {
  // configuration
  int device = 0;
  int flags = 0;
  int total_particles = 0;
  int cap_cells = 0;
  long long cap_voxels = 0;
  long long cap_samples = 0;
  // device state
  cudaStream_t stream = nullptr;
  DeviceState d{};
  SegParams *d_segs = nullptr;
  uint32_t *d_src_slot = nullptr;  // reorder scratch for key uploads
  void *d_prims = nullptr;         // voxeliser primitives
  int prim_cap = 0;
  void *d_mesh = nullptr;          // mesh voxeliser scratch (vertices, triangles, world vertices)
  size_t mesh_cap = 0;
  std::vector<SegParams> segs;
  bool segs_uploaded = false;
  size_t seg_capacity = 1;         // entries the device segment table holds
  int cseg_count = 0;              // entries of the constant table reserved (base in d.cseg_base)
  int pred_idx = 0;                // predicted positions live in pred_a (0) or pred_b (1)
  bool have_grid = false;          // keys / ids / offsets describe a built grid
  bool offsets_dirty = false;      // keys were uploaded; offsets follow on the next push
  bool keys_host_valid = false;
  std::vector<uint32_t> h_keys;    // host copy of uploaded keys (for offsets / checks)
  bool collider_installed = false;
  bool normal_zero = true;         // normal holds only the zeros it was created with
  bool normal_in_order = true;     // normal / delta still follow the slot order
  bool delta_in_order = true;
  bool next_normals_valid = false;  // normal_alt holds the normal pass of pred_cur() against the
                                    // current grid and parameters (left by the last fused
                                    // substep's XSPH pass)
  int collider_dims[3] = {0, 0, 0};
  std::string err;
  std::map<GraphKey, GraphEntry> graphs;
  std::vector<cudaEvent_t> events;

  int fail(int code, const std::string &msg);
  int cuda(cudaError_t e, const char *what);
  int check_launch(const char *what);
  int init_device();
  int allocate();
  void release();
  float4 *pred_cur();
  int set_push(const flowx_push *push);
  int upload_segs(const std::vector<SegParams> &s, int cells);
  // scatter + cell sort (x_order: cells by predicted x), or the reference's network
  void issue_cell_order(bool x_order);
  void issue_build_from_pred(const float4 *pred);
  int build_grid_generic();
  int issue_substep(int iterations, int pred_in_idx, bool normals_ready);
  bool segs_need_normal() const;
  void after_fused_substep();
  int ensure_grid();
  int ensure_offsets();
  int substep(int iterations);
  int step(int iterations, int substeps);
  int reorder_state(const std::vector<uint32_t> &src_slot);
  int profile_substeps(int iterations, int substeps, float *ms, int32_t *launches);
  // batched scenes
  bool batch = false;
  std::vector<long long> scene_voxels;  // collider voxels of each scene (0 = none)
  std::vector<char> scene_collider;     // collider installed per scene
  void drop_graphs();
};

}  // namespace flowx
