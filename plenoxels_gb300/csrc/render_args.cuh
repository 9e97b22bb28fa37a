// Validation of the plain-C grid and ray descriptors of include/plenoxels_gb300.h and
// their conversion into kernel arguments, shared by every entry point of the fused render
// kernels (capi.cu, noalloc.cu), so all of them accept the same arguments and launch the
// same kernels.
#pragma once

#include "pgb_host.h"
#include "render.cuh"

namespace pgb {

inline bool aligned(const void* p, uintptr_t a) { return ((uintptr_t)p % a) == 0; }

inline int check_grid(const pgb_grid* g) {
  if (!g || !g->cells) return PGB_ERR_ARG;
  if (g->dtype != PGB_F32 && g->dtype != PGB_BF16 && g->dtype != PGB_F64) return PGB_ERR_ARG;
  if (g->mode != PGB_NEAREST && g->mode != PGB_TRILINEAR) return PGB_ERR_ARG;
  for (int a = 0; a < 3; ++a)
    if (g->dims[a] <= 0) return PGB_ERR_ARG;
  const uint64_t cells = (uint64_t)g->dims[0] * g->dims[1] * g->dims[2];
  if (cells >= (1ull << 40)) return PGB_ERR_UNSUPPORTED;
  if (!aligned(g->cells, g->dtype == PGB_BF16 ? 8 : 16)) return PGB_ERR_ALIGN;
  return PGB_OK;
}

template <typename Real>
GridP<Real> grid_params(const pgb_grid* g) {
  GridP<Real> p = {};
  p.cells = g->cells;
  p.X = g->dims[0]; p.Y = g->dims[1]; p.Z = g->dims[2];
  p.fX = (Real)p.X; p.fY = (Real)p.Y; p.fZ = (Real)p.Z;
  p.ox = (Real)g->origin[0]; p.oy = (Real)g->origin[1]; p.oz = (Real)g->origin[2];
  p.pd = (Real)g->points_distance;
  p.clip = g->clip ? 1 : 0;
  p.alpha_floor = g->alpha_floor;
  return p;
}

inline int check_rays(const pgb_grid* g, const pgb_rays* r, bool need_target_or_cams) {
  if (!r || r->num_rays < 0 || r->num_samples < 0) return PGB_ERR_ARG;
  if (r->num_samples > kMaxSamples) return PGB_ERR_UNSUPPORTED;
  if (r->log_transmittance) {
    if (g->dtype == PGB_F64) return PGB_ERR_UNSUPPORTED;
    if (!g->clip) return PGB_ERR_ARG;  // log(1 - alpha) needs alpha in [0, 1]
  }
  if (r->cameras) {
    const pgb_cameras* c = r->cameras;
    if (g->dtype == PGB_F64) return PGB_ERR_UNSUPPORTED;
    if (!c->transforms || !c->images || c->num_cameras <= 0 || c->height <= 0 || c->width <= 0)
      return PGB_ERR_ARG;
    if (c->height != c->width) return PGB_ERR_UNSUPPORTED;
    if (!aligned(c->images, 16)) return PGB_ERR_ALIGN;
  } else if (r->num_rays > 0 && (!r->origins || !r->dirs)) {
    return PGB_ERR_ARG;
  }
  (void)need_target_or_cams;
  return PGB_OK;
}

template <typename Real>
RenderArgs<Real> render_args(const pgb_grid* g, const pgb_rays* r) {
  RenderArgs<Real> a = {};
  a.g = grid_params<Real>(g);
  a.origins = (const Real*)r->origins;
  a.dirs = (const Real*)r->dirs;
  if (r->cameras) {
    const pgb_cameras* c = r->cameras;
    a.use_cameras = 1;
    a.transforms = c->transforms;
    a.images = c->images;
    a.C = c->num_cameras;
    a.H = c->height;
    a.W = c->width;
    a.fov = c->camera_angle_x;
    a.near_dist = c->near;
    a.cam_seed = c->seed;
  }
  a.R = r->num_rays;
  a.S = r->num_samples;
  a.delta = (Real)r->delta_step;
  a.stratified = r->stratified ? 1 : 0;
  a.strat_seed = r->seed;
  a.first_ray = r->first_ray;
  a.grad_marks = r->grad_marks;
  a.term_thr = r->term_threshold;
  a.chunk_samples = r->chunk_samples;
  a.use_bg = r->use_background ? 1 : 0;
  for (int c = 0; c < 3; ++c) a.bg[c] = r->background[c];
  return a;
}

// The kernel arguments derived from the loss weights, in double on the host and rounded
// to Real once, as the kernel would round them.
template <typename Real>
void finish_args(RenderArgs<Real>& a) {
  a.use_beta = a.beta_w != 0.0 ? 1 : 0;
  a.grad_scale = (Real)(2.0 * a.loss_w * a.inv_count);
  // beta_w / (R*S) * (1 + 2 eps): the numerator of 1/(alpha+eps) + 1/(1-alpha+eps)
  a.beta_scale = (Real)(a.beta_w * a.inv_samples * (1.0 + 2.0 * (double)a.beta_eps));
}

template <typename Real>
int dispatch_render(const pgb_grid* g, const pgb_rays* r, RenderArgs<Real>& a, int phase,
                    cudaStream_t s);

template <>
inline int dispatch_render<float>(const pgb_grid* g, const pgb_rays* r, RenderArgs<float>& a, int phase,
                           cudaStream_t s) {
  finish_args(a);
  if (r->log_transmittance)
    return g->dtype == PGB_BF16 ? launch_render_logt_bf16(a, g->mode, phase, s)
                                : launch_render_logt_f32(a, g->mode, phase, s);
  return g->dtype == PGB_BF16 ? launch_render_bf16(a, g->mode, phase, s)
                              : launch_render_f32(a, g->mode, phase, s);
}
template <>
inline int dispatch_render<double>(const pgb_grid* g, const pgb_rays* r, RenderArgs<double>& a, int phase,
                            cudaStream_t s) {
  finish_args(a);
  (void)r;  // check_rays rejects the log-sum form for fp64 grids
  return launch_render_f64(a, g->mode, phase, s);
}


}  // namespace pgb
