// extern "C" entry points of include/plenoxels_gb300.h: argument validation, conversion
// of the plain-C descriptors into kernel arguments, and dispatch. Nothing here allocates
// or synchronises.
#include <atomic>
#include <cmath>

#include "pgb_host.h"
#include "render_args.cuh"

namespace pgb {

static std::atomic<int64_t> g_launches{0};

int after_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError() == cudaSuccess ? PGB_OK : PGB_ERR_LAUNCH;
}

// ops.cu
int op_generate_rays(const float*, int, int64_t, float, const float*, int, int, const float*, int,
                     float*, float*, int*, cudaStream_t);
int op_sample_points(const float*, int, int64_t, const float*, int, float, float*, cudaStream_t);
int op_coords_min(const float*, int64_t, float*, cudaStream_t);
int op_normalize(const float*, int64_t, const float*, float, float*, cudaStream_t);
int op_nearest_gather_f32(const GridP<float>&, int, const void*, int64_t, void*, uint8_t*, int64_t*, cudaStream_t);
int op_nearest_gather_f64(const GridP<double>&, const void*, int64_t, void*, uint8_t*, int64_t*, cudaStream_t);
int op_nearest_scatter_f32(const GridP<float>&, int, const void*, int64_t, const void*, void*, cudaStream_t);
int op_nearest_scatter_f64(const GridP<double>&, const void*, int64_t, const void*, void*, cudaStream_t);
int op_trilinear_gather_f32(const GridP<float>&, int, const void*, const int64_t*, int64_t, void*, int*, cudaStream_t);
int op_trilinear_gather_f64(const GridP<double>&, const void*, const int64_t*, int64_t, void*, int*, cudaStream_t);
int op_trilinear_scatter_f32(const GridP<float>&, int, const void*, const int64_t*, int64_t, const void*, void*, int*, cudaStream_t);
int op_trilinear_scatter_f64(const GridP<double>&, const void*, const int64_t*, int64_t, const void*, void*, int*, cudaStream_t);
int op_corner_indices(const void*, int, int64_t, int64_t*, cudaStream_t);
int op_grid_coords(const int[3], float, float*, int64_t*, cudaStream_t);
int op_gather_cells_f32(const GridP<float>&, int, const int64_t*, int64_t, void*, int*, cudaStream_t);
int op_gather_cells_f64(const GridP<double>&, const int64_t*, int64_t, void*, int*, cudaStream_t);
int op_scatter_cells_f32(const GridP<float>&, int, const int64_t*, int64_t, const void*, void*, int*, cudaStream_t);
int op_scatter_cells_f64(const GridP<double>&, const int64_t*, int64_t, const void*, void*, int*, cudaStream_t);
int op_in_bounds(const void*, int, int64_t, const int[3], uint8_t*, cudaStream_t);
int op_wrap(int64_t*, int64_t, const int[3], cudaStream_t);
int op_composite(const void*, int, int64_t, int, const void*, void*, int, cudaStream_t);
int composite_max_samples();
int op_render_indices_f32(const RenderArgs<float>&, int, int64_t*, uint8_t*, cudaStream_t);
int op_render_indices_f64(const RenderArgs<double>&, int, int64_t*, uint8_t*, cudaStream_t);
int op_render_coords_f32(const RenderArgs<float>&, float*, cudaStream_t);
int op_render_coords_f64(const RenderArgs<double>&, double*, cudaStream_t);
int op_fill_zero(void*, int64_t, cudaStream_t);
int op_clear_marked(void*, int, int64_t, uint32_t*, cudaStream_t);
int op_rgba_to_image(const float*, int, uint8_t*, cudaStream_t);

namespace {

template <typename Real>
int render_common(const pgb_grid* g, const pgb_rays* r, int phase, void* rgba_out,
                  const void* d_rgba, const void* target, double loss_w, void* grad,
                  void* loss_out, void* workspace, cudaStream_t s, double beta_w = 0.0,
                  float beta_eps = 0.f) {
  RenderArgs<Real> a = render_args<Real>(g, r);
  a.beta_w = beta_w;
  a.beta_eps = beta_eps;
  const double samples = (double)r->num_rays * (double)r->num_samples;
  a.inv_samples = samples > 0 ? 1.0 / samples : std::nan("");
  a.rgba_out = (Real*)rgba_out;
  a.d_rgba = (const Real*)d_rgba;
  a.target = (const Real*)target;
  a.grad = (Real*)grad;
  a.loss_out = (Real*)loss_out;
  if (workspace) {
    a.partials = (double*)workspace;
    a.partials_beta = (double*)workspace + kMaxTrainWarps;
    a.counter = (unsigned*)((char*)workspace + 2 * sizeof(double) * kMaxTrainWarps);
  }
  a.loss_w = loss_w;
  a.inv_count = r->num_rays > 0 ? 1.0 / (4.0 * (double)r->num_rays) : std::nan("");
  return dispatch_render<Real>(g, r, a, phase, s);
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_render_fwd(const pgb_grid* grid, const pgb_rays* rays, void* rgba_out, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if ((st = check_rays(grid, rays, false))) return st;
  if (rays->num_rays == 0) return PGB_OK;
  if (!rgba_out) return PGB_ERR_ARG;
  if (grid->dtype == PGB_F64)
    return render_common<double>(grid, rays, kForward, rgba_out, nullptr, nullptr, 1.0, nullptr,
                                 nullptr, nullptr, stream);
  return render_common<float>(grid, rays, kForward, rgba_out, nullptr, nullptr, 1.0, nullptr,
                              nullptr, nullptr, stream);
}

int pgb_render_bwd(const pgb_grid* grid, const pgb_rays* rays, const void* d_rgba,
                   void* grad_cells, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if ((st = check_rays(grid, rays, false))) return st;
  if (rays->num_rays == 0) return PGB_OK;
  if (!d_rgba || !grad_cells) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16)) return PGB_ERR_ALIGN;
  if (grid->dtype == PGB_F64)
    return render_common<double>(grid, rays, kBackward, nullptr, d_rgba, nullptr, 1.0, grad_cells,
                                 nullptr, nullptr, stream);
  return render_common<float>(grid, rays, kBackward, nullptr, d_rgba, nullptr, 1.0, grad_cells,
                              nullptr, nullptr, stream);
}

int64_t pgb_train_workspace_bytes(void) {
  return (int64_t)2 * sizeof(double) * kMaxTrainWarps + 256;
}

int pgb_render_train(const pgb_grid* grid, const pgb_rays* rays, const void* target,
                     double loss_weight, void* rgba_out, void* grad_cells, void* loss_out,
                     void* workspace, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if ((st = check_rays(grid, rays, true))) return st;
  if (!grad_cells || !loss_out || !workspace) return PGB_ERR_ARG;
  if (!rays->cameras && rays->num_rays > 0 && !target) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16) || !aligned(workspace, 16)) return PGB_ERR_ALIGN;
  if (grid->dtype == PGB_F64)
    return render_common<double>(grid, rays, kTrain, rgba_out, nullptr, target, loss_weight,
                                 grad_cells, loss_out, workspace, stream);
  return render_common<float>(grid, rays, kTrain, rgba_out, nullptr, target, loss_weight,
                              grad_cells, loss_out, workspace, stream);
}

int pgb_render_train_terms(const pgb_grid* grid, const pgb_rays* rays, const void* target,
                           const pgb_loss_terms* terms, void* rgba_out, void* grad_cells,
                           void* losses_out, void* workspace, pgb_stream_t stream) {
  if (!terms) return PGB_ERR_ARG;
  int st = check_grid(grid);
  if (st) return st;
  if ((st = check_rays(grid, rays, true))) return st;
  if (!grad_cells || !losses_out || !workspace) return PGB_ERR_ARG;
  if (!rays->cameras && rays->num_rays > 0 && !target) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16) || !aligned(workspace, 16)) return PGB_ERR_ALIGN;
  if (grid->dtype == PGB_F64)
    return render_common<double>(grid, rays, kTrain, rgba_out, nullptr, target, terms->mse_weight,
                                 grad_cells, losses_out, workspace, stream, terms->beta_weight,
                                 terms->beta_eps);
  return render_common<float>(grid, rays, kTrain, rgba_out, nullptr, target, terms->mse_weight,
                              grad_cells, losses_out, workspace, stream, terms->beta_weight,
                              terms->beta_eps);
}

int pgb_render_sample_indices(const pgb_grid* grid, const pgb_rays* rays, int64_t* index_out,
                              uint8_t* inbounds_out, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if ((st = check_rays(grid, rays, false))) return st;
  if (rays->num_rays == 0 || rays->num_samples == 0) return PGB_OK;
  if (!index_out && !inbounds_out) return PGB_ERR_ARG;
  if (grid->dtype == PGB_F64) {
    RenderArgs<double> a = render_args<double>(grid, rays);
    return op_render_indices_f64(a, grid->mode, index_out, inbounds_out, stream);
  }
  RenderArgs<float> a = render_args<float>(grid, rays);
  return op_render_indices_f32(a, grid->mode, index_out, inbounds_out, stream);
}

int pgb_render_sample_coords(const pgb_grid* grid, const pgb_rays* rays, void* coords_out,
                             pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if ((st = check_rays(grid, rays, false))) return st;
  if (rays->num_rays == 0 || rays->num_samples == 0) return PGB_OK;
  if (!coords_out) return PGB_ERR_ARG;
  if (grid->dtype == PGB_F64)
    return op_render_coords_f64(render_args<double>(grid, rays), (double*)coords_out, stream);
  return op_render_coords_f32(render_args<float>(grid, rays), (float*)coords_out, stream);
}

int pgb_generate_rays(const float* transforms, int32_t num_cameras, int64_t rays_per_camera,
                      float camera_angle_x, const float* images, int32_t height, int32_t width,
                      const float* uv, int32_t even_spread, float* dirs_out, float* pixels_out,
                      int32_t* status_out, pgb_stream_t stream) {
  if (num_cameras < 0 || rays_per_camera < 0 || height <= 0 || width <= 0) return PGB_ERR_ARG;
  if ((int64_t)num_cameras * rays_per_camera == 0) return PGB_OK;
  if (!transforms || !images || !dirs_out || !pixels_out) return PGB_ERR_ARG;
  if (!aligned(images, 16) || !aligned(pixels_out, 16)) return PGB_ERR_ALIGN;
  int side = 0;
  if (even_spread) {
    side = (int)std::llround(std::sqrt((double)rays_per_camera));
    if ((int64_t)side * side != rays_per_camera) return PGB_ERR_ARG;
  } else if (!uv) {
    return PGB_ERR_ARG;
  }
  if ((int64_t)num_cameras * rays_per_camera == 0) return PGB_OK;
  return op_generate_rays(transforms, num_cameras, rays_per_camera, camera_angle_x, images, height,
                          width, even_spread ? nullptr : uv, side, dirs_out, pixels_out, status_out,
                          stream);
}

int pgb_sample_points(const float* transforms, int32_t num_cameras, int64_t rays_per_camera,
                      const float* dirs, int32_t num_samples, float delta_step, float* samples_out,
                      pgb_stream_t stream) {
  if (num_cameras < 0 || rays_per_camera < 0 || num_samples < 0) return PGB_ERR_ARG;
  if ((int64_t)num_cameras * rays_per_camera * num_samples == 0) return PGB_OK;
  if (!transforms || !dirs || !samples_out) return PGB_ERR_ARG;
  return op_sample_points(transforms, num_cameras, rays_per_camera, dirs, num_samples, delta_step,
                          samples_out, stream);
}

int pgb_coords_min(const float* coords, int64_t count, float* min_out, pgb_stream_t stream) {
  if (!coords || !min_out || count <= 0) return PGB_ERR_ARG;
  return op_coords_min(coords, count, min_out, stream);
}

int pgb_normalize_samples(const float* samples, int64_t count, const float* grid_min,
                          float points_distance, float* out, pgb_stream_t stream) {
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!samples || !grid_min || !out) return PGB_ERR_ARG;
  return op_normalize(samples, count, grid_min, points_distance, out, stream);
}

int pgb_nearest_gather(const pgb_grid* grid, const void* normalized, int64_t count, void* vals_out,
                       uint8_t* inbounds_out, int64_t* index_out, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!normalized || !vals_out) return PGB_ERR_ARG;
  if (grid->dtype == PGB_F64)
    return op_nearest_gather_f64(grid_params<double>(grid), normalized, count, vals_out,
                                 inbounds_out, index_out, stream);
  return op_nearest_gather_f32(grid_params<float>(grid), grid->dtype == PGB_BF16, normalized, count,
                               vals_out, inbounds_out, index_out, stream);
}

int pgb_nearest_scatter(const pgb_grid* grid, const void* normalized, int64_t count,
                        const void* d_vals, void* grad_cells, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!normalized || !d_vals || !grad_cells) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16)) return PGB_ERR_ALIGN;
  if (grid->dtype == PGB_F64)
    return op_nearest_scatter_f64(grid_params<double>(grid), normalized, count, d_vals, grad_cells,
                                  stream);
  return op_nearest_scatter_f32(grid_params<float>(grid), grid->dtype == PGB_BF16, normalized, count,
                                d_vals, grad_cells, stream);
}

int pgb_grid_coords(const int32_t dims[3], float points_distance, float* coords_out,
                    int64_t* meshgrid_out, pgb_stream_t stream) {
  if (!dims || (!coords_out && !meshgrid_out)) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  const int d[3] = {dims[0], dims[1], dims[2]};
  return op_grid_coords(d, points_distance, coords_out, meshgrid_out, stream);
}

int pgb_gather_cells(const pgb_grid* grid, const int64_t* indices, int64_t count, void* vals_out,
                     int32_t* status_out, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!indices || !vals_out) return PGB_ERR_ARG;
  if (grid->dtype == PGB_F64)
    return op_gather_cells_f64(grid_params<double>(grid), indices, count, vals_out, status_out, stream);
  return op_gather_cells_f32(grid_params<float>(grid), grid->dtype == PGB_BF16, indices, count,
                             vals_out, status_out, stream);
}

int pgb_scatter_cells(const pgb_grid* grid, const int64_t* indices, int64_t count,
                      const void* d_vals, void* grad_cells, int32_t* status_out,
                      pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!indices || !d_vals || !grad_cells) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16)) return PGB_ERR_ALIGN;
  if (grid->dtype == PGB_F64)
    return op_scatter_cells_f64(grid_params<double>(grid), indices, count, d_vals, grad_cells,
                                status_out, stream);
  return op_scatter_cells_f32(grid_params<float>(grid), grid->dtype == PGB_BF16, indices, count,
                              d_vals, grad_cells, status_out, stream);
}

int pgb_corner_indices(const void* normalized, int32_t dtype, int64_t count, int64_t* corners_out,
                       pgb_stream_t stream) {
  if (count < 0 || (dtype != PGB_F32 && dtype != PGB_F64)) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!normalized || !corners_out) return PGB_ERR_ARG;
  return op_corner_indices(normalized, dtype == PGB_F64, count, corners_out, stream);
}

int pgb_in_bounds(const void* indices, int32_t index_kind, int64_t count, const int32_t dims[3],
                  uint8_t* out, pgb_stream_t stream) {
  if (count < 0 || !dims) return PGB_ERR_ARG;
  if (index_kind != PGB_INDEX_F32 && index_kind != PGB_INDEX_F64 && index_kind != PGB_INDEX_I64)
    return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!indices || !out) return PGB_ERR_ARG;
  const int d[3] = {dims[0], dims[1], dims[2]};
  return op_in_bounds(indices, index_kind, count, d, out, stream);
}

int pgb_wrap_indices(int64_t* indices, int64_t count, const int32_t dims[3], pgb_stream_t stream) {
  if (!dims || count < 0) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!indices) return PGB_ERR_ARG;
  const int d[3] = {dims[0], dims[1], dims[2]};
  return op_wrap(indices, count, d, stream);
}

int pgb_trilinear_gather(const pgb_grid* grid, const void* normalized, const int64_t* corners,
                         int64_t count, void* out, int32_t* status_out, pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!normalized || !corners || !out) return PGB_ERR_ARG;
  if (grid->dtype == PGB_F64)
    return op_trilinear_gather_f64(grid_params<double>(grid), normalized, corners, count, out,
                                   status_out, stream);
  return op_trilinear_gather_f32(grid_params<float>(grid), grid->dtype == PGB_BF16, normalized,
                                 corners, count, out, status_out, stream);
}

int pgb_trilinear_scatter(const pgb_grid* grid, const void* normalized, const int64_t* corners,
                          int64_t count, const void* d_out, void* grad_cells, int32_t* status_out,
                          pgb_stream_t stream) {
  int st = check_grid(grid);
  if (st) return st;
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!normalized || !corners || !d_out || !grad_cells) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16)) return PGB_ERR_ALIGN;
  if (grid->dtype == PGB_F64)
    return op_trilinear_scatter_f64(grid_params<double>(grid), normalized, corners, count, d_out,
                                    grad_cells, status_out, stream);
  return op_trilinear_scatter_f32(grid_params<float>(grid), grid->dtype == PGB_BF16, normalized,
                                  corners, count, d_out, grad_cells, status_out, stream);
}

int pgb_composite_fwd(const void* samples, int32_t dtype, int64_t num_rays, int32_t num_samples,
                      void* out, pgb_stream_t stream) {
  if (num_rays < 0 || num_samples < 0) return PGB_ERR_ARG;
  if (dtype != PGB_F32 && dtype != PGB_F64) return PGB_ERR_ARG;
  if (num_samples > composite_max_samples()) return PGB_ERR_UNSUPPORTED;
  if (num_rays == 0) return PGB_OK;
  if (!out || (num_samples > 0 && !samples)) return PGB_ERR_ARG;
  if (!aligned(samples, 16)) return PGB_ERR_ALIGN;
  return op_composite(samples, dtype == PGB_F64, num_rays, num_samples, nullptr, out, 0, stream);
}

int pgb_composite_bwd(const void* samples, int32_t dtype, int64_t num_rays, int32_t num_samples,
                      const void* d_out, void* d_samples, pgb_stream_t stream) {
  if (num_rays < 0 || num_samples < 0) return PGB_ERR_ARG;
  if (dtype != PGB_F32 && dtype != PGB_F64) return PGB_ERR_ARG;
  if (num_samples > composite_max_samples()) return PGB_ERR_UNSUPPORTED;
  if (num_rays == 0 || num_samples == 0) return PGB_OK;
  if (!samples || !d_out || !d_samples) return PGB_ERR_ARG;
  if (!aligned(samples, 16)) return PGB_ERR_ALIGN;
  return op_composite(samples, dtype == PGB_F64, num_rays, num_samples, d_out, d_samples, 1, stream);
}

int pgb_rgba_to_image(const float* rgba, int32_t res, uint8_t* image_out, pgb_stream_t stream) {
  if (res < 0) return PGB_ERR_ARG;
  if (res == 0) return PGB_OK;
  if (!rgba || !image_out) return PGB_ERR_ARG;
  return op_rgba_to_image(rgba, res, image_out, stream);
}

int pgb_fill_zero(void* ptr, int64_t bytes, pgb_stream_t stream) {
  if (bytes < 0) return PGB_ERR_ARG;
  if (bytes == 0) return PGB_OK;
  if (!ptr) return PGB_ERR_ARG;
  if (!aligned(ptr, 16)) return PGB_ERR_ALIGN;
  return op_fill_zero(ptr, bytes, stream);
}

int64_t pgb_mark_words(int64_t num_cells) { return num_cells > 0 ? mark_words(num_cells) : 0; }

int pgb_clear_marked(void* grad_cells, int32_t cell_bytes, int64_t num_cells, uint32_t* grad_marks,
                     pgb_stream_t stream) {
  if (num_cells < 0 || (cell_bytes != 16 && cell_bytes != 32)) return PGB_ERR_ARG;
  if (num_cells == 0) return PGB_OK;
  if (!grad_cells || !grad_marks) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16) || !aligned(grad_marks, 4)) return PGB_ERR_ALIGN;
  return op_clear_marked(grad_cells, cell_bytes, num_cells, grad_marks, stream);
}

float pgb_hash_uniform(uint64_t seed, uint64_t a, uint32_t b) {
  return hash_to_unit(hash_stream(seed, a), b);
}

int64_t pgb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

const char* pgb_version(void) { return "plenoxels_gb300 0.1.0 (sm_103a)"; }

const char* pgb_status_string(int status) {
  switch (status) {
    case PGB_OK: return "ok";
    case PGB_ERR_ARG: return "invalid argument";
    case PGB_ERR_ALIGN: return "misaligned pointer";
    case PGB_ERR_LAUNCH: return "kernel launch failed";
    case PGB_ERR_UNSUPPORTED: return "unsupported configuration";
    default: return "unknown status";
  }
}

}  // extern "C"
