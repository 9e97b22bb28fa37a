/*
 * plenoxels_gb300 — C ABI of the GB300 (sm_103a) differentiable voxel-grid renderer.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream, launches
 * asynchronously on that stream, allocates nothing, and returns PGB_OK (0) or a
 * negative PGB_ERR_* code for an argument or launch error. No entry point
 * synchronises the device. Each entry point names the reference function it
 * replaces (paths are relative to the DanJbk/Plenoxels repository).
 *
 * Grid layout (src/grid_functions.py:184-217 generate_grid): a dense, contiguous,
 * channels-last [X, Y, Z, 4] tensor of interleaved R, G, B, alpha cells. Cell
 * (i, j, k) sits at world position origin + (i, j, k) * points_distance, where
 * origin is the per-axis minimum of the reference's grid coordinate table
 * ((1 - ceil(s/2)) * points_distance).
 *
 * Storage types: PGB_F32 (16 B cells), PGB_BF16 (8 B cells, fp32 arithmetic and fp32
 * gradients) and PGB_F64 (32 B cells, fp64 arithmetic; used for finite-difference
 * checks). "Real" below means float for F32/BF16 grids and double for F64 grids.
 */
#ifndef PLENOXELS_GB300_H
#define PLENOXELS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* pgb_stream_t;

enum {
  PGB_OK = 0,
  PGB_ERR_ARG = -1,         /* null pointer, bad size, bad enum */
  PGB_ERR_ALIGN = -2,       /* a pointer is not aligned for vector cell access */
  PGB_ERR_LAUNCH = -3,      /* the CUDA launch itself failed */
  PGB_ERR_UNSUPPORTED = -4  /* valid but unsupported combination (e.g. too many samples) */
};

enum { PGB_F32 = 0, PGB_BF16 = 1, PGB_F64 = 2 };
enum { PGB_NEAREST = 0, PGB_TRILINEAR = 1 };

/* A dense channels-last RGBA voxel grid. */
typedef struct {
  const void* cells;        /* [X,Y,Z,4] of dtype; 16-byte aligned (8 for BF16) */
  int32_t dtype;            /* PGB_F32 | PGB_BF16 | PGB_F64 */
  int32_t dims[3];          /* X, Y, Z */
  double origin[3];         /* world position of cell (0,0,0), held exactly in "Real" */
  double points_distance;   /* cell pitch, held exactly in "Real" */
  int32_t clip;             /* 1: clamp cell values to [0,1] at lookup (scripts/train.py:146) */
  int32_t mode;             /* PGB_NEAREST | PGB_TRILINEAR */
  float alpha_floor;        /* >0: after the clamp, alpha below this reads as 0 (the inference
                               threshold of src/visualization.py:117-119); 0 for training */
} pgb_grid;

/* Cameras for in-kernel ray generation (src/ray_sampling.py:195-264). */
typedef struct {
  const float* transforms;  /* [C,4,4] camera-to-world; columns x, y, back, position */
  const float* images;      /* [C,H,W,4] RGBA target pixels */
  int32_t num_cameras;      /* C */
  int32_t height, width;    /* H, W (square images only, as the reference indexes them) */
  float camera_angle_x;     /* horizontal field of view, used linearly (ray_sampling.py:234) */
  float near;               /* rays start at position + near * direction */
  uint64_t seed;            /* pixel-position RNG seed (counter-based hash; see pgb_hash_uniform) */
} pgb_cameras;

/* A batch of rays and how each ray is sampled (src/ray_sampling.py:128-169). */
typedef struct {
  const void* origins;      /* [R,3] Real: first point of each ray (NULL when cameras != NULL) */
  const void* dirs;         /* [R,3] Real: unit directions (NULL when cameras != NULL) */
  const pgb_cameras* cameras; /* host pointer; non-NULL: rays generated in-kernel, camera-major */
  int64_t num_rays;         /* R */
  int32_t num_samples;      /* S: samples at t_k = delta_step * k, k = 1..S */
  double delta_step;        /* held exactly in "Real" */
  int32_t stratified;       /* 1: t_k = delta_step * (k - j_k), j_k in [0,1) from the hash */
  uint64_t seed;            /* stratification seed */
  float term_threshold;     /* >0: stop a ray once its transmittance falls below this */
  int32_t use_background;   /* 1: output rgb += (1 - alpha) * background (alpha unchanged) */
  float background[3];      /* e.g. 1,1,1 for a white background; the reference has none */
  int32_t log_transmittance; /* 1: T = exp(compensated sum of log(1 - alpha)) instead of the
                                reference's product; fp32/BF16 grids with clip only (the
                                precision form; no counterpart in the reference) */
  int32_t chunk_samples;    /* samples a warp gathers between transmittance checks: 0 picks
                               automatically, else 32, 64, 128, 256 or 512 (raised when a ray
                               would span more than 32 chunks). With clip on (and no beta
                               term), a ray stops after the chunk in which its transmittance
                               reaches exactly 0, once the samples behind the opaque sample
                               can no longer change a gradient (its own alpha gradient is
                               masked by the clamp, or a second opaque sample was read):
                               results are unchanged and the rest of the ray is never read.
                               Tuning only. */
  int64_t first_ray;        /* index of this batch's first ray in the stratification stream
                               (0 for a batch of its own): ranks that split one batch of
                               explicit rays pass their share's offset, and every ray is
                               sampled as in the unsplit batch */
  uint32_t* grad_marks;     /* optional device bitmap (NULL: none) of the gradient's 4-cell
                               units, pgb_mark_words(cells) words: the backward and training
                               entry points set bit (c/4) % 32 of word c/128 for every
                               gradient cell c they write, so pgb_clear_marked can re-zero
                               just those units. No counterpart in the reference. */
} pgb_rays;

/* ---- fused render path (scripts/train.py:142-156 composed with src/ray_sampling.py,
 *      src/grid_functions.py; one warp per ray, no per-sample intermediates) ---- */

/* Forward: rgba_out[R,4] = composited premultiplied RGB and accumulated alpha.
 * Replaces sample_camera_rays_batched -> normalize_samples_for_indecies ->
 * get_nearest_voxels | trilinear_interpolation -> *mask -> compute_alpha_weighted_pixels
 * (scripts/train.py:130-151). */
int pgb_render_fwd(const pgb_grid* grid, const pgb_rays* rays, void* rgba_out, pgb_stream_t stream);

/* Backward of pgb_render_fwd: accumulates dL/dcells into grad_cells ([X,Y,Z,4], fp32 for
 * F32/BF16 grids, fp64 for F64), which the caller zeroes first. Replaces the autograd
 * replay of loss.backward() (scripts/train.py:181). */
int pgb_render_bwd(const pgb_grid* grid, const pgb_rays* rays, const void* d_rgba,
                   void* grad_cells, pgb_stream_t stream);

/* Fused training step: forward, MSE against target (mean over R*4 entries times
 * loss_weight, scripts/train.py:156), and backward in one launch. target is [R,4] Real
 * (ignored when rays->cameras is set: targets are the sampled image pixels).
 * rgba_out may be NULL. loss_out[0] receives the loss (Real), written by the kernel:
 * any address the GPU can store to, device memory or pinned host memory (under unified
 * addressing a pinned host pointer is a device pointer), so a host reads the loss after
 * the stream synchronises with no copy. workspace must hold pgb_train_workspace_bytes()
 * bytes and be zeroed once before first use; the kernel leaves it zeroed again. */
int pgb_render_train(const pgb_grid* grid, const pgb_rays* rays, const void* target,
                     double loss_weight, void* rgba_out, void* grad_cells, void* loss_out,
                     void* workspace, pgb_stream_t stream);
int64_t pgb_train_workspace_bytes(void);

/* No counterpart in the reference: pgb_render_train for callers that cannot allocate
 * device memory (their device memory is owned by another allocator, or they run a loop
 * that must not allocate). Same arguments and results as pgb_render_train minus the
 * workspace: the loss-reduction scratch is a fixed array inside the library (about 32 KiB per
 * device, held by every GPU that loads the library until the process exits). It calls no
 * cudaMalloc, cudaFree or other allocating routine.
 * - At most PGB_NOALLOC_MAX_RAYS rays per call; more returns PGB_ERR_UNSUPPORTED.
 * - The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 *   for that device; make that first call before any stream capture.
 * - Every call shares the array: calls that overlap on the GPU (other streams, other host
 *   threads) race on it. Each call clears the counter it needs on its own stream. */
enum { PGB_NOALLOC_MAX_RAYS = 32768 };
int pgb_render_train_noalloc(const pgb_grid* grid, const pgb_rays* rays, const void* target,
                             double loss_weight, void* rgba_out, void* grad_cells, void* loss_out,
                             pgb_stream_t stream);

/* pgb_render_train with the reference's extra loss terms (scripts/train.py:156, :170-177):
 * loss = mse_weight * MSE + beta_weight * mean over all R*S samples of
 * log(alpha + beta_eps) - log(1 - alpha + beta_eps) (alpha after the clip and the mask).
 * losses_out[0] receives the weighted MSE and, when beta_weight != 0, losses_out[1] the
 * weighted beta term (Real). Same workspace as pgb_render_train. */
typedef struct {
  double mse_weight;
  double beta_weight;
  float beta_eps;
} pgb_loss_terms;
int pgb_render_train_terms(const pgb_grid* grid, const pgb_rays* rays, const void* target,
                           const pgb_loss_terms* terms, void* rgba_out, void* grad_cells,
                           void* losses_out, void* workspace, pgb_stream_t stream);

/* Debug/parity view of the fused kernels' own index math: for every sample of every
 * ray, the wrapped cell indices the lookup reads (nearest: [R,S,3]; trilinear:
 * [R,S,8,3], corner order of src/grid_functions.py:16-24) and the in-bounds flag
 * [R,S]. index_out is int64. */
int pgb_render_sample_indices(const pgb_grid* grid, const pgb_rays* rays, int64_t* index_out,
                              uint8_t* inbounds_out, pgb_stream_t stream);
/* The normalised coordinates (position - origin) / points_distance of every sample of
 * every ray, as the fused kernels compute them (src/ray_sampling.py:161-167, :12-13):
 * coords_out [R,S,3] Real. */
int pgb_render_sample_coords(const pgb_grid* grid, const pgb_rays* rays, void* coords_out,
                             pgb_stream_t stream);

/* ---- batched form: many scenes, one persistent launch per training step ----
 * Scenes of different sizes, each a dense [X,Y,Z,4] grid (BF16 or fp32 cells) whose
 * unoccupied cells are zero and are not parameters, with a brick mask for empty-space
 * skipping; rays of all scenes in one queue. The step is the fused training step of
 * scripts/train.py:130-181 for every ray of every scene. No counterpart in the reference
 * beyond that composition (the reference trains one scene, densely). */
typedef struct {
  const void* cells;        /* [X,Y,Z,4], dtype of the batch */
  const uint32_t* bricks;   /* dilated brick mask (pgb_build_bricks) or NULL: no skipping */
  const uint32_t* occupancy;/* cell bits (bit c of word c/32) or NULL: every cell is a parameter */
  void* grad_cells;         /* [X,Y,Z,4] fp32 gradient, written only at occupied cells */
  int32_t dims[3];          /* X, Y, Z */
  int32_t brick_log2;       /* bricks are 2^brick_log2 cells per axis */
  int32_t brick_dims[3];    /* ceil(dims / 2^brick_log2) */
  float origin[3];          /* world position of cell (0,0,0) */
  float points_distance;
  int32_t num_samples;      /* samples per ray of this scene */
  float delta_step;
} pgb_scene;

/* Dilated brick mask of a scene from its per-cell occupancy bits (bit c of word c/32 for
 * cell c = (i*Y + j)*Z + k): bit b of bricks_out is set when brick b or any of its seven
 * upper neighbours (+1 in any subset of axes) holds an occupied cell, so a sample whose
 * floor corner lies in a clear brick reads only unoccupied cells. bricks_out must hold
 * ceil(prod(brick_dims)/32) words and is overwritten. */
int pgb_build_bricks(const uint32_t* cell_bits, const int32_t dims[3], int32_t brick_log2,
                     uint32_t* bricks_out, pgb_stream_t stream);

/* Packs a uint8/bool mask of count entries into bits (bit c of word c/32). No counterpart
 * in the reference (batched form). */
int pgb_pack_mask(const uint8_t* mask, int64_t count, uint32_t* bits_out, pgb_stream_t stream);

/* No counterpart in the reference (batched form). Zeroes the gradients of all scenes of
 * a device-resident scene table: the occupied
 * cells where a scene has an occupancy mask (the only cells the step writes), every cell
 * otherwise. max_cells bounds the largest scene. */
int pgb_batch_zero_grads(const pgb_scene* scenes, int32_t num_scenes, int64_t max_cells,
                         pgb_stream_t stream);

/* No counterpart in the reference (batched form; per ray it is scripts/train.py:130-181).
 * One training step over all rays: ray r belongs to scene ray_scene[r] and starts at
 * origins[r] along dirs[r]; target[r] is its pixel. scenes is a DEVICE array of
 * num_scenes (<= 256) descriptors. Gradients accumulate into each scene's grad_cells;
 * loss_out[0] = loss_weight * mean over all rays and channels of the squared error.
 * term_threshold > 0 stops a ray once its transmittance falls below it (checked every
 * 32*slots_per_lane samples). slots_per_lane in {1,2,4,8} and threads_per_block in
 * {128,256} are the tile choices (0: defaults); a ray spans at most 32 chunks, so every
 * scene needs num_samples <= 1024 * slots_per_lane (a longer ray's loss and RGBA come
 * back NaN). merge_updates = 1 (trilinear) sums the updates that lanes of a warp make to
 * the same cell before the atomic adds (a tile choice: same gradient, summed in another
 * order). workspace: pgb_batch_workspace_bytes(R), zeroed once before first use; the
 * call's two kernels (the persistent step, then the ordered loss sum) leave their
 * counters zeroed. */
int64_t pgb_batch_workspace_bytes(int64_t num_rays);
int pgb_batch_train(const pgb_scene* scenes, int32_t num_scenes, int32_t dtype, int32_t mode,
                    int32_t clip, const float* origins, const float* dirs, const float* target,
                    const int32_t* ray_scene, int64_t num_rays, float term_threshold,
                    int32_t stratified, uint64_t seed, double loss_weight, float* rgba_out,
                    float* loss_out, void* workspace, int32_t slots_per_lane,
                    int32_t threads_per_block, int32_t merge_updates, pgb_stream_t stream);

/* ---- optimiser side of the training step (scripts/train.py:44-65, :89, :163-184) ---- */

/* TV sum of squares of a dense fp32 [X,Y,Z,4] grid: sumsq_out[0] (device fp64) = sum over
 * all axis-neighbour pairs and channels of (v_i - v_j)^2; tv_loss = sqrt(sumsq)
 * (scripts/train.py:44-65). Deterministic. workspace: pgb_tv_workspace_bytes(), zeroed
 * once; left zeroed. */
int64_t pgb_tv_workspace_bytes(void);
int pgb_tv_sumsq(const float* cells, const int32_t dims[3], double* sumsq_out, void* workspace,
                 pgb_stream_t stream);
/* grad += weight / sqrt(sumsq) * sum over neighbours j of (v_i - v_j): the gradient of
 * weight * sqrt(sumsq) (scripts/train.py:163-165). No-op when sumsq == 0. */
int pgb_tv_grad(const float* cells, const int32_t dims[3], const double* sumsq, float weight,
                float* grad_cells, pgb_stream_t stream);
/* One torch.optim.Adam step (scripts/train.py:89, :182; no weight decay, no amsgrad) over
 * count fp32 values (count % 4 == 0, 16-byte aligned): exp_avg = lerp(exp_avg, grad,
 * 1 - beta1), exp_avg_sq = beta2 * exp_avg_sq + (1 - beta2) * grad^2, param -= lr / bc1 *
 * exp_avg / (sqrt(exp_avg_sq) / sqrt(bc2) + eps), bc_i = 1 - beta_i^step; then
 * abs_grad_accum += |grad| (scripts/train.py:184, optional) and grad = 0 when zero_grad. */
int pgb_adam_step(float* param, float* grad, float* exp_avg, float* exp_avg_sq,
                  float* abs_grad_accum, int64_t count, double lr, double beta1, double beta2,
                  double eps, int64_t step, int32_t zero_grad, pgb_stream_t stream);
/* pgb_adam_step on grad + the gradient of tv_weight * sqrt(Q) (Q from pgb_tv_sumsq of
 * param_in, the TV term of scripts/train.py:44-65, :163-165), the stencil evaluated as
 * pgb_tv_grad does, in the same pass as the update: the TV gradient pass and the Adam pass
 * of scripts/train.py:163-165, :182 fused. param_in is the [X,Y,Z,4] grid before the step,
 * param_out (a different buffer) receives it after; the moments, the accumulator and the
 * cleared gradient are updated in place. No counterpart in the reference (it runs TV
 * backward and optimizer.step() as separate passes). */
int pgb_adam_tv_step(const float* param_in, float* param_out, float* grad, float* exp_avg,
                     float* exp_avg_sq, float* abs_grad_accum, const int32_t dims[3],
                     const double* tv_sumsq, float tv_weight, double lr, double beta1, double beta2,
                     double eps, int64_t step, int32_t zero_grad, pgb_stream_t stream);

/* src/grid_functions.py:173-181 average_pool3d_grid (scripts/train.py:108-123): average of
 * a cubic window of `window` cells, stride `stride`, no padding, of a contiguous fp32
 * [X,Y,Z,4] grid into [Xo,Yo,Zo,4], Xo = (X - window) / stride + 1. pgb_avg_pool3d_shape
 * gives the output dims and the scratch bytes both directions need (caller-provided). */
int pgb_avg_pool3d_shape(const int32_t dims[3], int32_t window, int32_t stride,
                         int32_t out_dims[3], int64_t* scratch_bytes);
int pgb_avg_pool3d_fwd(const float* cells, const int32_t dims[3], int32_t window, int32_t stride,
                       void* scratch, float* out, pgb_stream_t stream);
/* Adjoint (autograd of F.avg_pool3d at src/grid_functions.py:178): d_cells[X,Y,Z,4] = the
 * pooled gradient spread back over each window (every cell written, so no prior zeroing
 * is needed). */
int pgb_avg_pool3d_bwd(const float* d_out, const int32_t dims[3], int32_t window, int32_t stride,
                       void* scratch, float* d_cells, pgb_stream_t stream);

/* ---- drop-in operators, one per reference function ---- */

/* src/ray_sampling.py:195-264 generate_rays_batched. uv: [C*Rc,2] uniforms in [0,1)
 * (the reference's torch.rand draw), or NULL with even_spread=1 (linspace grid of
 * side x side rays, side*side == Rc). Writes dirs_out[C*Rc,3], pixels_out[C*Rc,4].
 * status_out (optional device int32) is OR-ed with 1 when a pixel index falls outside
 * the image (the reference raises IndexError there); that ray's pixel is zero. */
int pgb_generate_rays(const float* transforms, int32_t num_cameras, int64_t rays_per_camera,
                      float camera_angle_x, const float* images, int32_t height, int32_t width,
                      const float* uv, int32_t even_spread, float* dirs_out, float* pixels_out,
                      int32_t* status_out, pgb_stream_t stream);

/* src/ray_sampling.py:159-167: samples_out[C*Rc*S,3] = position(camera(r)) +
 * dirs[r] * (delta_step * k), k = 1..S. transforms gives the camera positions. */
int pgb_sample_points(const float* transforms, int32_t num_cameras, int64_t rays_per_camera,
                      const float* dirs, int32_t num_samples, float delta_step,
                      float* samples_out, pgb_stream_t stream);

/* src/ray_sampling.py:13, the grid_indices.min(0) reduction: min_out[3] (device). */
int pgb_coords_min(const float* coords, int64_t count, float* min_out, pgb_stream_t stream);

/* src/ray_sampling.py:12-13 normalize_samples_for_indecies:
 * out = (samples - grid_min) / points_distance with IEEE division. grid_min is device [3]. */
int pgb_normalize_samples(const float* samples, int64_t count, const float* grid_min,
                          float points_distance, float* out, pgb_stream_t stream);

/* src/grid_functions.py:103-114 get_nearest_voxels (with :47-63 and :66-79):
 * round half to even, in-bounds flag, periodic wrap, gather. normalized is [N,3] Real.
 * vals_out [N,4] Real, inbounds_out [N] (0/1), index_out [N,3] int64 (optional). */
int pgb_nearest_gather(const pgb_grid* grid, const void* normalized, int64_t count,
                       void* vals_out, uint8_t* inbounds_out, int64_t* index_out,
                       pgb_stream_t stream);
/* Backward of pgb_nearest_gather (the index backward that loss.backward() at
 * scripts/train.py:181 runs through src/grid_functions.py:114): grad_cells[idx] += d_vals
 * (clip mask applied). */
int pgb_nearest_scatter(const pgb_grid* grid, const void* normalized, int64_t count,
                        const void* d_vals, void* grad_cells, pgb_stream_t stream);

/* src/grid_functions.py:184-217 generate_grid: world coordinates coords_out [X,Y,Z,3]
 * fp32 = (index - ceil(dim/2) + 1) * points_distance and the integer index table
 * meshgrid_out [X,Y,Z,3] int64 (either may be NULL). */
int pgb_grid_coords(const int32_t dims[3], float points_distance, float* coords_out,
                    int64_t* meshgrid_out, pgb_stream_t stream);

/* src/grid_functions.py:154-170 (the gather of collect_cell_information_via_indices):
 * vals_out[M,4] = cells[idx[m]] for int64 indices [M,3]. Negative indices count from the
 * end; an index outside the grid OR-s 1 into status_out and yields zeros. */
int pgb_gather_cells(const pgb_grid* grid, const int64_t* indices, int64_t count, void* vals_out,
                     int32_t* status_out, pgb_stream_t stream);
/* Backward of pgb_gather_cells (autograd of the gather at src/grid_functions.py:169):
 * grad_cells[idx[m]] += d_vals[m] (clip mask applied). */
int pgb_scatter_cells(const pgb_grid* grid, const int64_t* indices, int64_t count,
                      const void* d_vals, void* grad_cells, int32_t* status_out,
                      pgb_stream_t stream);

/* src/grid_functions.py:220-246 get_grid_points_indices: corners_out [N,8,3] int64. */
int pgb_corner_indices(const void* normalized, int32_t dtype, int64_t count,
                       int64_t* corners_out, pgb_stream_t stream);

/* src/grid_functions.py:47-63 find_out_of_bound on float or int64 indices [N,3]. */
int pgb_in_bounds(const void* indices, int32_t index_kind, int64_t count, const int32_t dims[3],
                  uint8_t* out, pgb_stream_t stream);
enum { PGB_INDEX_F32 = 0, PGB_INDEX_F64 = 1, PGB_INDEX_I64 = 2 };

/* src/grid_functions.py:66-79 fix_out_of_bounds: in-place floor-mod of [M,3] int64. */
int pgb_wrap_indices(int64_t* indices, int64_t count, const int32_t dims[3], pgb_stream_t stream);

/* src/grid_functions.py:7-44 trilinear_interpolation: out[N,4] Real from the already
 * wrapped corners [N,8,3] int64 and frac(normalized). grid->clip applies the clamp.
 * Negative corner indices count from the end (torch indexing); a corner outside the
 * grid is skipped and OR-s 1 into status_out (optional device int32), where the
 * reference raises IndexError. */
int pgb_trilinear_gather(const pgb_grid* grid, const void* normalized, const int64_t* corners,
                         int64_t count, void* out, int32_t* status_out, pgb_stream_t stream);
/* Backward of pgb_trilinear_gather into grad_cells (autograd of the gathers and blends of
 * src/grid_functions.py:31-42). */
int pgb_trilinear_scatter(const pgb_grid* grid, const void* normalized, const int64_t* corners,
                          int64_t count, const void* d_out, void* grad_cells,
                          int32_t* status_out, pgb_stream_t stream);

/* src/ray_sampling.py:172-192 compute_alpha_weighted_pixels over [M,S,4] samples
 * (M = cameras * rays). out[M,4] = (sum w*rgb, sum w), w_k = a_k * prod_{j<k}(1 - a_j). */
int pgb_composite_fwd(const void* samples, int32_t dtype, int64_t num_rays, int32_t num_samples,
                      void* out, pgb_stream_t stream);
/* Backward (autograd of src/ray_sampling.py:181-188): d_samples[M,S,4] from d_out[M,4]
 * (division-free, exact at alpha == 1). */
int pgb_composite_bwd(const void* samples, int32_t dtype, int64_t num_rays, int32_t num_samples,
                      const void* d_out, void* d_samples, pgb_stream_t stream);

/* ---- utilities ---- */

/* Image of the premultiplied RGBA of res x res even-spread rays (src/visualization.py:
 * 147-152): u8 = clip(round_half_even(255 * rgba), 0, 255), stored transposed, so
 * image_out[a][b] is ray b * res + a. */
int pgb_rgba_to_image(const float* rgba, int32_t res, uint8_t* image_out, pgb_stream_t stream);

/* ---- previews and clean-up (src/visualization.py:157-232, src/grid_functions.py:260-280) ---- */

/* Width xs of the splat preview of a camera (host transform, row-major 4x4) of height
 * size_y: int(size_y * |x axis| / |y axis|), fp32 as the reference computes it. */
int pgb_splat_size(const float* transform, int32_t size_y, int32_t* width_out);
/* Point-splat preview (visulize_3d_in_2d_fast): every cell of a contiguous fp32
 * [X,Y,Z,4] grid with alpha > alpha_min projects to a pixel of an [xs, size_y] image; the
 * nearest such cell paints its RGB, other pixels are white. transform is a HOST pointer.
 * keys_scratch holds xs * size_y uint64; image_out is [xs, size_y, 3] fp32. */
int pgb_splat_preview(const float* cells, const int32_t dims[3], float points_distance,
                      const float* transform, float camera_angle_x, int32_t size_y, float alpha_min,
                      unsigned long long* keys_scratch, float* image_out, pgb_stream_t stream);
/* convolve_grid_to_remove_noise on a contiguous fp32 [X,Y,Z,4] grid, in place: `repeats`
 * times, every cell whose summed neighbour alpha over the filled ball (kernel_size^3,
 * offsets with distance <= radius, centre excluded, zero padding) is below threshold is
 * cleared. kernel_size odd and <= 7; sums_scratch holds X*Y*Z floats. */
int pgb_remove_noise(float* cells, const int32_t dims[3], int32_t kernel_size, double radius,
                     float threshold, int32_t repeats, float* sums_scratch, pgb_stream_t stream);

/* Zero `bytes` bytes at ptr (16-byte aligned) with a vectorised store kernel: the
 * gradient zeroing of optimizer.zero_grad() (scripts/train.py:180) and of a fresh .grad. */
int pgb_fill_zero(void* ptr, int64_t bytes, pgb_stream_t stream);
/* Words of the gradient mark bitmap (pgb_rays.grad_marks) of num_cells cells. */
int64_t pgb_mark_words(int64_t num_cells);
/* Zeroes the gradient units marked in grad_marks (pgb_rays.grad_marks: 4 cells per unit,
 * pgb_mark_words(num_cells) words) and clears the marks. A dense gradient buffer whose only writes since
 * it was last zero are marked steps is zero again afterwards: the zeroing of
 * optimizer.zero_grad() (scripts/train.py:180) restricted to the cells a step wrote. cell
 * bytes: 16 (F32/BF16 grids' fp32 gradient) or 32 (F64). No counterpart in the reference. */
int pgb_clear_marked(void* grad_cells, int32_t cell_bytes, int64_t num_cells, uint32_t* grad_marks,
                     pgb_stream_t stream);

/* The counter-based uniform in [0,1) used for stratification and in-kernel ray
 * generation, evaluated on the host: uniform(seed, a, b). Exact multiples of 2^-24. No
 * counterpart in the reference (it draws torch.rand; the drop-in generate_rays_batched
 * still does). */
float pgb_hash_uniform(uint64_t seed, uint64_t a, uint32_t b);

/* Library utilities, no counterpart in the reference: kernels launched in this process
 * (all entry points), the version string and the text of a status code. */
int64_t pgb_launch_count(void);
const char* pgb_version(void);
const char* pgb_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* PLENOXELS_GB300_H */
