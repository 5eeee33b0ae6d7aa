/* flowx.h - C ABI of the GB300 PBF substep library (libflowx.so).
 *
 * Drop-in for the GPU compute path of Flow-X's solver: the Blender `gpu`
 * compute plumbing of solver/gpu_util.py plus the pass sequencing of
 * solver/sph.py. Every entry point takes plain pointers and sizes, returns an
 * int status (FLOWX_OK = 0) and never traps; the text of the last failure is
 * available from flowx_last_error().
 *
 * Ownership and ordering: device memory belongs to the context; host buffers
 * belong to the caller. A context is used from one thread at a time. All work
 * is ordered on the context's CUDA stream; flowx_download() and
 * flowx_splat() with a host destination return after the data has arrived.
 *
 * Buffer layouts at this boundary are the reference's (solver/sph.py:127-152,
 * solver/gpu_util.py:28-59), indexed by particle id, as flat arrays without
 * the reference's 256-wide texture padding:
 *   POSITIONS, VELOCITIES, PREDICTED, DELTA, NORMAL   N x float4
 *   LAMBDA                                             N x float4 (density, lambda, 0, 0)
 *   KEYS                                               S x float4 (cell key, particle id, 0, 0),
 *                                                      S = next power of two >= N; slots >= N
 *                                                      are padding (key = cell count)
 *   CELL_START, CELL_END                               C x float, -1 for an empty cell
 *   SURFACE                                            samples x float (flowx_splat)
 * A download may also ask for fewer bytes than the whole buffer: it then
 * returns the first ones.
 */
#ifndef FLOWX_H
#define FLOWX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FLOWX_ABI_VERSION 1

/* Status codes. */
enum {
  FLOWX_OK = 0,
  FLOWX_ERR_ARG = 1,      /* bad argument, size or layout */
  FLOWX_ERR_CUDA = 2,     /* a CUDA call failed (text in flowx_last_error) */
  FLOWX_ERR_STATE = 3,    /* call not valid in the context's current state */
  FLOWX_ERR_CAPACITY = 4, /* larger than the context was created for */
};

/* The 128-byte push-constant block, field for field
 * (shaders/sph_common.glsl:10-17, packed by solver/sph.py:433-461):
 *   i_layout   = (particle_count, tex_width, tex_width, sorted_count)
 *   i_grid     = (cells_x, cells_y, cells_z, cell_count)
 *   i_sort     = (bitonic_k, bitonic_j, floatBitsToInt(scorr_k), floatBitsToInt(surface_tension))
 *                for the splat: (samples_x, samples_y, samples_z, floatBitsToInt(spacing))
 *                (shaders/surface_splat.glsl:14)
 *   f_lo       = (domain_min.xyz, cell_size)
 *   f_hi       = (domain_max.xyz, particle_radius); for the splat: (surface_lo.xyz, 0)
 *   f_sph      = (smoothing_radius, particle_mass, rest_density, relaxation_epsilon);
 *                for the splat f_sph.x is the surface kernel radius
 *   f_sim      = (viscosity, dt, gravity, boundary_damping)
 *   i_collider = (collider_dims.xyz, floatBitsToInt(collider_voxel_size)); voxel 0 = none
 * The bitonic (k, j) lanes and the texture widths are accepted and ignored. */
typedef struct flowx_push {
  int32_t i_layout[4];
  int32_t i_grid[4];
  int32_t i_sort[4];
  float f_lo[4];
  float f_hi[4];
  float f_sph[4];
  float f_sim[4];
  int32_t i_collider[4];
} flowx_push;

/* Buffer ids (the images of solver/sph.py:127-152 and the splat grid). */
enum {
  FLOWX_BUF_POSITIONS = 0,
  FLOWX_BUF_VELOCITIES = 1,
  FLOWX_BUF_LAMBDA = 2,
  FLOWX_BUF_PREDICTED = 3,
  FLOWX_BUF_DELTA = 4,
  FLOWX_BUF_NORMAL = 5,
  FLOWX_BUF_KEYS = 6,
  FLOWX_BUF_CELL_START = 7,
  FLOWX_BUF_CELL_END = 8,
  FLOWX_BUF_SURFACE = 9,
};

/* Pass ids, numbered as solver/sph.py:_PASSES (154-167) plus the splat.
 * GRID_KEY, SORT, CELL_CLEAR and CELL_RANGE are not separate passes here:
 * flowx_build_grid() does all four. */
enum {
  FLOWX_PASS_NORMAL = 0,
  FLOWX_PASS_PREDICT = 1,
  FLOWX_PASS_GRID_KEY = 2,
  FLOWX_PASS_SORT = 3,
  FLOWX_PASS_CELL_CLEAR = 4,
  FLOWX_PASS_CELL_RANGE = 5,
  FLOWX_PASS_LAMBDA = 6,
  FLOWX_PASS_DELTA = 7,
  FLOWX_PASS_APPLY_DELTA = 8,
  FLOWX_PASS_VELOCITY = 9,
  FLOWX_PASS_XSPH = 10,
  FLOWX_PASS_FINALIZE = 11,
};

/* Context flags. */
enum {
  /* The fused substep also writes the XSPH velocity correction to DELTA, as
   * the reference's sph_xsph.glsl leaves it (off by default: nothing in the
   * substep reads it back). */
  FLOWX_FLAG_KEEP_DELTA = 1,
  /* The fused substep evaluates the reference's float expressions operation
   * for operation (bit-identical to a float32 evaluation without FMA
   * contraction). Without it, pair terms are re-associated for throughput
   * (FMA, one reciprocal square root per pair), within float32 rounding. The
   * per-pass API (flowx_run_pass) is always exact. */
  FLOWX_FLAG_EXACT = 2,
  /* Every grid build orders the particles inside each cell the way the
   * reference's own grid build does: the bitonic compare-exchange network of
   * sph_sort.glsl over the sph_grid_key.glsl array, driven as
   * solver/sph.py:488-495 drives it (unstable, by cell key only). Sorted keys,
   * cell ranges and membership are the same as without the flag; only the
   * order inside a cell, and so the order neighbour sums visit, changes. With
   * FLOWX_FLAG_EXACT the substep then reproduces the reference's passes
   * in the reference's own visiting order. Costs the network's
   * log2(S)(log2(S)+1)/2 steps per build; single-scene contexts only. */
  FLOWX_FLAG_REFERENCE_ORDER = 4,
  /* The fused substep's neighbour passes run one warp per particle (its
   * lanes test 32 candidates at once) or one thread per particle. Results
   * are bit-identical either way. Without either flag the library takes one
   * warp per particle up to FLOWX_WARP_PASSES_MAX_PARTICLES particles, where
   * one thread per particle leaves most of the GPU idle (measured on a GB300:
   * 3.3x faster substeps at 3,200 particles, 1.25x at 20,000, 0.7x at
   * 38,400), and one thread per particle above. */
  FLOWX_FLAG_WARP_PASSES = 8,
  FLOWX_FLAG_THREAD_PASSES = 16,
};
#define FLOWX_WARP_PASSES_MAX_PARTICLES 25000

/* Sizes a context is created for (solver/sph.py:350-369 _allocate). */
typedef struct flowx_config {
  int32_t particle_count;       /* N, fixed for the context's lifetime */
  int32_t max_cells;            /* capacity for i_grid.w */
  int64_t max_collider_voxels;  /* capacity of the collider grid */
  int64_t max_surface_samples;  /* capacity of the splat grid */
  int32_t device;               /* CUDA device ordinal */
  int32_t flags;                /* FLOWX_FLAG_* */
} flowx_config;

/* An analytic collider shape for flowx_voxelize(): kind 0 = sphere (a =
 * centre, r = radius), 1 = axis-aligned box (a = min, b = max), 2 = vertical
 * cylinder (a = base centre, r = radius, b[2] = top). */
typedef struct flowx_primitive {
  int32_t kind;
  int32_t pad;
  double a[3];
  double b[3];
  double r;
} flowx_primitive;

typedef struct flowx_ctx flowx_ctx;

/* Create / destroy a context. Replaces solver/sph.py:350-369 (_allocate) and
 * the texture creation of solver/gpu_util.py:46-59 (make_texture). After
 * creation every buffer is zero and the positions of a fresh context must be
 * uploaded before stepping. */
int flowx_create(const flowx_config *config, flowx_ctx **out);
int flowx_destroy(flowx_ctx *ctx);

/* Text of the last failure on this context (or of the last failed
 * flowx_create when ctx is NULL). Never NULL. */
const char *flowx_last_error(const flowx_ctx *ctx);

/* Host -> device copy of a whole buffer in the reference layout (see the file
 * header). Replaces solver/gpu_util.py:46-59 (make_texture with values).
 * Uploading KEYS re-orders the context's particle state to that key order;
 * the keys must be sorted by cell with ids forming a permutation of 0..N-1.
 * CELL_START / CELL_END are checked against the uploaded keys. */
int flowx_upload(flowx_ctx *ctx, int buffer, const void *host, size_t bytes);

/* Device -> host copy in the reference layout. Replaces
 * solver/gpu_util.py:62-89 (read_texture, read_scalar_texture). */
int flowx_download(flowx_ctx *ctx, int buffer, void *host, size_t bytes);

/* Install the collider occupancy grid (uint8, x fastest, origin at the
 * domain's low corner, nonzero = occupied). Replaces the R32F collider texture
 * of collision/__init__.py:276-290 read as "> 0.5" (sph_common.glsl:154-160).
 * occupancy NULL or voxel_size 0 removes it. */
int flowx_set_collider(flowx_ctx *ctx, const uint8_t *occupancy, const int32_t dims[3], float voxel_size);

/* Build the collider grid on the device from analytic shapes (centre-inside
 * test in double precision). Same layout as flowx_set_collider. No reference
 * counterpart: the reference voxelises meshes on the CPU
 * (collision/__init__.py:304-367). */
int flowx_voxelize(flowx_ctx *ctx, const flowx_primitive *prims, int count, const int32_t dims[3],
                   float voxel_size, const float origin[3]);

/* One triangle-mesh collider for flowx_voxelize_meshes(): local-space
 * vertices (vertex_count x 3 floats), triangles (triangle_count x 3 vertex
 * indices) and the object's world matrix (4 x 4, row-major, applied to column
 * vectors: world = M [v; 1], Blender's matrix_world). */
typedef struct flowx_mesh {
  const float *vertices;
  int32_t vertex_count;
  const int32_t *triangles;
  int32_t triangle_count;
  float matrix_world[16];
} flowx_mesh;

/* Build the collider grid on the device from triangle meshes: a voxel is
 * occupied when its centre is inside any mesh, by the parity of the mesh's
 * crossings of the vertical ray above the centre, each mesh marking only the
 * voxels of its world bounding box's index range; a mesh with a singular
 * matrix marks nothing. Replaces collision/__init__.py:304-367
 * (_rebuild_grid, _point_inside: BVH ray casts on the CPU) and the union of
 * :225-242; crossings are counted exactly in double precision with
 * watertight edge tests rather than by Blender's ray casts. Same layout as
 * flowx_set_collider; triangle indices outside [0, vertex_count) are
 * rejected before anything runs. */
int flowx_voxelize_meshes(flowx_ctx *ctx, const flowx_mesh *meshes, int count, const int32_t dims[3],
                          float voxel_size, const float origin[3]);

/* Read back the installed collider grid (the flowx_set_collider layout, one
 * byte per voxel, 1 = occupied): the occupancy collision/__init__.py keeps on
 * the CPU for its viewport overlay (ColliderGrid.occupancy). bytes must equal
 * the installed grid's voxel count; waits for the copy. */
int flowx_download_collider(flowx_ctx *ctx, uint8_t *host, size_t bytes);

/* The neighbour grid from the current predicted positions: keys, cell ranges
 * and the particle order. Replaces solver/sph.py:482-498 (_build_grid: the
 * grid-key pass, the bitonic (k, j) dispatch loop, cell clear, cell range). */
int flowx_build_grid(flowx_ctx *ctx, const flowx_push *push);

/* One substep with `iterations` Jacobi iterations. Replaces
 * solver/sph.py:501-514 (_substep); the normal pass runs when the block's
 * surface tension is > 0, as there. */
int flowx_substep(flowx_ctx *ctx, const flowx_push *push, int iterations);

/* `substeps` substeps as one CUDA-graph launch (captured on first use for a
 * given shape). Replaces the substep loop of solver/sph.py:517-530 (_step).
 * A single-scene context's graphs carry the scene's parameters, so a push
 * block whose values differ from the previous call's (dt, h, ...) re-captures
 * them; an unchanged push block reuses them. */
int flowx_step(flowx_ctx *ctx, const flowx_push *push, int iterations, int substeps);

/* One reference pass on the current buffers, as one gpu.compute.dispatch of
 * solver/gpu_util.py:157-159 (dispatch_1d) of that pass would. */
int flowx_run_pass(flowx_ctx *ctx, int pass_id, const flowx_push *push);

/* The per-frame density splat with the splat's push block (see flowx_push).
 * Replaces solver/surface.py:201-240 (update: dispatch + read_scalar_texture).
 * host_out may be NULL to keep the grid on the device (download SURFACE). */
int flowx_splat(flowx_ctx *ctx, const flowx_push *splat_push, float *host_out, size_t bytes);

/* Wait for all queued work. */
int flowx_synchronize(flowx_ctx *ctx);

/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or events against it. */
int flowx_get_stream(flowx_ctx *ctx, void **stream);

/* Device time in milliseconds of `steps` flowx_step() calls (graph launches),
 * measured with CUDA events on the context's stream after one untimed warm-up
 * launch. No reference counterpart (the reference times whole frames on the
 * host, solver/sph.py:517-545). */
int flowx_time_steps(flowx_ctx *ctx, const flowx_push *push, int iterations, int substeps, int steps,
                     float *ms);

/* Per-kernel device time: runs `substeps` substeps launch by launch with CUDA
 * events around every kernel and accumulates milliseconds and launch counts
 * per kernel id into ms[] / launches[] (arrays of flowx_kernel_count()
 * entries; names from flowx_kernel_name()). No reference counterpart. */
int flowx_profile_substeps(flowx_ctx *ctx, const flowx_push *push, int iterations, int substeps, float *ms,
                           int32_t *launches);
int flowx_kernel_count(void);
const char *flowx_kernel_name(int kernel_id);

/* Total number of kernel launches this library has issued (all contexts). */
int64_t flowx_launch_count(void);

/* ---- batched scenes -------------------------------------------------------
 * No reference counterpart: the reference simulates one domain per scene
 * (README.md:141). A batch is a context created for the summed particle,
 * cell and collider-voxel counts of several independent scenes; every kernel
 * of the substep then serves all scenes in one launch. Particle buffers
 * (flowx_upload / flowx_download) are the scenes' arrays concatenated in scene
 * order; downloaded keys carry the batch-global cell index. */

/* Install the scenes, one push block each (particle count, grid, parameters,
 * collider dims / voxel). The counts must sum to the context's particle
 * count. Single-scene entry points (flowx_substep, flowx_step, ...) are then
 * refused; use the batch ones. The kernels read the scenes' parameters from
 * a 128-entry constant-memory table per device, which the process's batches
 * share (a slice each, first come, first served, returned on destroy); a
 * batch that finds no room reads them from device memory instead: the same
 * results, a few percent slower. */
int flowx_batch_set_scenes(flowx_ctx *ctx, const flowx_push *pushes, int nscenes);

/* Where a scene lives in the concatenated arrays. */
int flowx_batch_scene_range(flowx_ctx *ctx, int scene, int32_t *first_particle, int32_t *particle_count,
                            int32_t *first_cell, int32_t *cell_count);

/* Collider occupancy of one scene (layout of flowx_set_collider); dims and
 * voxel must match the scene's push block. */
int flowx_batch_set_collider(flowx_ctx *ctx, int scene, const uint8_t *occupancy, const int32_t dims[3],
                             float voxel_size);

/* Grid build, one substep, or `substeps` substeps as one CUDA-graph launch,
 * for all scenes at once (each with its own dt and parameters). */
int flowx_batch_build_grid(flowx_ctx *ctx);
int flowx_batch_substep(flowx_ctx *ctx, int iterations);
int flowx_batch_step(flowx_ctx *ctx, int iterations, int substeps);

/* The density splat of one scene, with that scene's splat push block. */
int flowx_batch_splat(flowx_ctx *ctx, int scene, const flowx_push *splat_push, float *host_out, size_t bytes);

/* ---- launch shapes ----------------------------------------------------------
 * Block sizes per kernel: flowx_autotune times the fused substep launch by
 * launch with candidate sizes (64, 128, 256, 512) on the context's current
 * state, restoring that state after every trial, and keeps the fastest per
 * kernel; chosen (flowx_kernel_count() entries, may be NULL) receives the
 * result, 0 meaning the kernel's default. `push` is ignored for a batch.
 * flowx_set_block_sizes installs sizes directly. No reference counterpart. */
int flowx_autotune(flowx_ctx *ctx, const flowx_push *push, int iterations, int32_t *chosen);
int flowx_set_block_sizes(flowx_ctx *ctx, const int32_t *blocks);

/* ---- Differentiable substeps (no reference counterpart) -------------------
 * A checkpointed forward of the fused substep (solver/sph.py:501-514, the
 * same float32 expressions as FLOWX_FLAG_EXACT) and its hand-written adjoint.
 * Particle arrays here are DEVICE pointers (N x float4, particle-id order) on
 * the object's stream. The neighbour grid of every substep is held fixed
 * (not differentiated); the state entering each substep is checkpointed and
 * the Jacobi iterates are recomputed during the adjoint. The first substep
 * sees the state the reference's _allocate and _seed leave (sph.py:350-369,
 * :606): predicted = positions, densities zero, grid built from positions. */
typedef struct flowx_adjoint flowx_adjoint;

typedef struct flowx_adjoint_config {
  int32_t particle_count;
  int32_t max_cells;
  int32_t max_substeps;        /* substeps one forward may record */
  int32_t max_iterations;      /* Jacobi iterations per substep, >= 1 */
  int64_t max_collider_voxels;
  int64_t max_surface_samples; /* splat grid capacity, 0 = no splat */
  int32_t device;
  int32_t reserved;
} flowx_adjoint_config;

int flowx_adjoint_create(const flowx_adjoint_config *config, flowx_adjoint **out);
int flowx_adjoint_destroy(flowx_adjoint *adj);
const char *flowx_adjoint_last_error(const flowx_adjoint *adj);
int flowx_adjoint_get_stream(flowx_adjoint *adj, void **stream);
/* Collider occupancy (host bytes, the flowx_set_collider layout). */
int flowx_adjoint_set_collider(flowx_adjoint *adj, const uint8_t *occupancy, const int32_t dims[3], float voxel_size);
/* `substeps` substeps with `iterations` Jacobi iterations from (positions,
 * velocities); writes the final state to positions_out / velocities_out and,
 * when splat_push is not NULL, the density splat of the final positions
 * (flowx_splat's values) to surface. Records what flowx_substep_adjoint needs. */
int flowx_adjoint_forward(flowx_adjoint *adj, const flowx_push *push, int iterations, int substeps,
                          const float *positions, const float *velocities, float *positions_out,
                          float *velocities_out, const flowx_push *splat_push, float *surface);
/* Reverse mode over the substeps of the last flowx_adjoint_forward: given the
 * cotangents of the surface (NULL = zero), the final positions and the final
 * velocities (NULL = zero), writes the gradients with respect to the initial
 * positions and velocities (N x float4 each, w lanes zero). */
int flowx_substep_adjoint(flowx_adjoint *adj, const float *surface_grad, const float *positions_out_grad,
                          const float *velocities_out_grad, float *positions_grad, float *velocities_grad);

/* ---- Marching cubes (solver/marching_cubes.py:191-280, extract) ----------
 * Iso-surface of a float32 lattice field on the device (x fastest, sample
 * (i, j, k) at origin + (i, j, k) * spacing, inside where value >= iso), as
 * the reference's indexed mesh: the same vertices in the same order with the
 * same float64 coordinates, and the same triangles. The object owns its
 * device scratch and mesh buffers (grown as needed). */
typedef struct flowx_mc flowx_mc;

int flowx_mc_create(int32_t device, flowx_mc **out);
int flowx_mc_destroy(flowx_mc *mc);
const char *flowx_mc_last_error(const flowx_mc *mc);
/* Extract on `stream` (NULL = default stream; it is synchronised for the
 * counts). field: device pointer, dims[0] * dims[1] * dims[2] floats. The
 * stream must stay valid until flowx_mc_download / flowx_mc_mesh of this
 * extraction (they order on it); flowx_mc_destroy does not use it. */
int flowx_mc_extract(flowx_mc *mc, const float *field, const int32_t dims[3], const double origin[3], double spacing,
                     double iso, void *stream, int64_t *vertex_count, int64_t *triangle_count);
/* The last extraction to host: vertices V x 3 doubles, triangles T x 3 int32. */
int flowx_mc_download(flowx_mc *mc, double *vertices, size_t vertex_bytes, int32_t *triangles,
                      size_t triangle_bytes);
/* Device pointers to the last extraction's mesh (valid until the next extract). */
int flowx_mc_mesh(flowx_mc *mc, const double **vertices, const int32_t **triangles);
/* The derived case table (no GPU needed): triangle_count triangles of edge
 * indices for corner-sign case mc_case (bit c = corner c inside); edges must
 * hold 15 ints. */
int flowx_mc_case_table(int32_t mc_case, int32_t *edges, int32_t *triangle_count);
/* The context's splat grid on the device (after flowx_splat), for
 * flowx_mc_extract: the pointer and its capacity in samples. */
int flowx_surface_field(flowx_ctx *ctx, const float **field, int64_t *samples);

/* ---- Disk cache (solver/cache.py, format FLWXCA01 version 2) -------------
 * Per-frame (positions, velocities) snapshots in the reference's file layout
 * (header, then frames seed_frame + 1 .. last_frame of N x 4 f32 positions
 * and N x 4 f32 velocities at arithmetic offsets; last_frame rewritten after
 * every frame write). Which file to trust (config hash, collider names) is
 * the host's decision, as in the reference; these calls read and write. */
typedef struct flowx_cache flowx_cache;

typedef struct flowx_cache_header {
  char flowx_version[16];        /* NUL padded */
  int32_t particle_count;
  int32_t seed_frame;
  int32_t last_frame;            /* output of flowx_cache_info; create sets it to seed_frame */
  float fps;
  int32_t collider_count;
  const char *const *collider_names;  /* create: collider_count names; info: NULL (see below) */
  uint8_t config_hash[32];       /* sha256 of the run's settings */
} flowx_cache_header;

/* A new file (truncated) holding only the header. */
int flowx_cache_create(const char *path, const flowx_cache_header *header, flowx_cache **out);
/* An existing file; FLOWX_ERR_ARG when it is not a version-2 FLWXCA01 file. */
int flowx_cache_open(const char *path, flowx_cache **out);
int flowx_cache_close(flowx_cache *cache);
const char *flowx_cache_last_error(const flowx_cache *cache);
int flowx_cache_info(const flowx_cache *cache, flowx_cache_header *header);
const char *flowx_cache_collider_name(const flowx_cache *cache, int32_t index);
/* solver/cache.py:339-379: store a context's positions and velocities (id
 * order) as `frame`; frames at or before the seed frame are not stored. */
int flowx_cache_write_frame(flowx_cache *cache, flowx_ctx *ctx, int32_t frame);
/* solver/cache.py:382-421 + solver/sph.py:700-733: install a cached frame in
 * the context (positions, velocities, predicted = positions, lambda zero, the
 * grid rebuilt with `push`). FLOWX_ERR_ARG outside seed_frame < frame <=
 * last_frame. */
int flowx_cache_load_frame(flowx_cache *cache, flowx_ctx *ctx, int32_t frame, const flowx_push *push);
/* The same with host arrays (N x 4 floats each), no device involved. */
int flowx_cache_write_frame_host(flowx_cache *cache, int32_t frame, const float *positions, const float *velocities);
int flowx_cache_read_frame_host(flowx_cache *cache, int32_t frame, float *positions, float *velocities);

/* Grid build that allocates nothing. There is no counterpart in the
 * reference: its grid build (solver/sph.py:482-498) always runs inside a
 * context that owns its buffers.
 *
 * For callers that cannot let a library allocate device memory: an
 * application that reserves its device-memory budget up front and hands out
 * pieces of it, or code in a region where the device-wide synchronisation of
 * cudaMalloc / cudaFree is not allowed. No context: all arguments are device
 * pointers owned by the caller.
 *   predicted    particle_count x float4, predicted positions in id order
 *   keys         key_count x float4 out, key_count >= particle_count; the KEYS
 *                layout above (padding slots get (cell count, slot))
 *   cell_start,  C x float out each, C = push->i_grid[3]; -1 for an empty
 *   cell_end     cell (the CELL_START / CELL_END layouts above)
 *   stream       cudaStream_t the work is ordered on (NULL = default stream)
 * The result equals flowx_build_grid's for the same predicted positions and
 * push block. Returns without waiting for the GPU.
 *
 * Scratch is one static device array of the library, sized for at most
 * 65536 particles and 262144 cells; larger sizes return FLOWX_ERR_CAPACITY.
 * The first call made with a device current is a warm-up: it looks the
 * array's address up for that device and, with lazy module loading, is
 * where the runtime loads the module, which reserves the array and may
 * synchronise the device. Make it at set-up, before any stream capture;
 * later calls allocate nothing. The address is kept for the process: do not
 * use the library after a cudaDeviceReset. Every call clears the cell
 * counters (the only scratch that must start at zero) itself. All calls on a
 * device share the scratch, so calls whose GPU work overlaps race: issue
 * them on one stream and from one host thread at a time (each call enqueues
 * several launches; two threads' sequences on one stream can interleave).
 * The message of a failure is returned by flowx_build_grid_static_error
 * (per host thread). */
int flowx_build_grid_static(const float *predicted, int32_t particle_count, const flowx_push *push, float *keys,
                            int32_t key_count, float *cell_start, float *cell_end, void *stream);
const char *flowx_build_grid_static_error(void);

#ifdef __cplusplus
}
#endif

#endif /* FLOWX_H */
