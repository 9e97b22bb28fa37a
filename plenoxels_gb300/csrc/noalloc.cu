// The fused training step for callers that cannot allocate device memory.
//
// pgb_render_train needs a caller-provided workspace for its loss reduction (one
// partial per block and a block counter). Some callers cannot call cudaMalloc: a host
// whose device memory is owned by another allocator (a framework's caching allocator or
// a pre-reserved pool that hands out no extra buffers), or a loop that must not allocate
// once it runs (a real-time render or training loop with a fixed memory budget). For
// them this file keeps that scratch in a fixed device array that is part of the loaded
// library, so the call needs only the inputs and outputs.
#include <cmath>
#include <mutex>
#include <type_traits>

#include "pgb_host.h"
#include "render.cuh"

namespace pgb {
namespace {

// One ray per warp, so a call of at most PGB_NOALLOC_MAX_RAYS rays launches at most
// kNoAllocMaxBlocks blocks, each writing one loss partial.
constexpr int kNoAllocWarpsPerBlock = kRenderThreads / kWarp;
constexpr int kNoAllocMaxBlocks = PGB_NOALLOC_MAX_RAYS / kNoAllocWarpsPerBlock;
static_assert(PGB_NOALLOC_MAX_RAYS % kNoAllocWarpsPerBlock == 0, "ray limit must fill whole blocks");
static_assert(kNoAllocMaxBlocks * kNoAllocWarpsPerBlock <= kMaxTrainWarps,
              "the train launcher must not cap the grid below one ray per warp");
constexpr size_t kCounterOffset = (size_t)kNoAllocMaxBlocks * sizeof(double);
constexpr size_t kScratchBytes = kCounterOffset + 256;

// The scratch: block loss partials, then the block counter. Every GPU that loads the
// library holds it until the process exits; every call shares it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_scratch_mutex;
void* g_scratch_address[64] = {};  // device address of g_noalloc_scratch, per device

// Device address of the scratch on the current device. The array's name in host code is
// a host-side stand-in, not a device address; the address comes from
// cudaGetSymbolAddress, once per device, with that device current.
int scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PGB_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_address[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr)
      return PGB_ERR_LAUNCH;
    g_scratch_address[dev] = p;
  }
  *out = g_scratch_address[dev];
  return PGB_OK;
}

inline bool aligned_to(const void* p, uintptr_t a) { return ((uintptr_t)p % a) == 0; }

template <typename Real>
int launch_noalloc(const pgb_grid* g, const pgb_rays* r, const void* target, double loss_weight,
                   void* rgba_out, void* grad_cells, void* loss_out, unsigned char* scratch,
                   cudaStream_t stream) {
  RenderArgs<Real> a = {};
  a.g.cells = g->cells;
  a.g.X = g->dims[0]; a.g.Y = g->dims[1]; a.g.Z = g->dims[2];
  a.g.fX = (Real)a.g.X; a.g.fY = (Real)a.g.Y; a.g.fZ = (Real)a.g.Z;
  a.g.ox = (Real)g->origin[0]; a.g.oy = (Real)g->origin[1]; a.g.oz = (Real)g->origin[2];
  a.g.pd = (Real)g->points_distance;
  a.g.clip = g->clip ? 1 : 0;
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
  a.term_thr = r->term_threshold;
  a.use_bg = r->use_background ? 1 : 0;
  for (int c = 0; c < 3; ++c) a.bg[c] = r->background[c];
  a.rgba_out = (Real*)rgba_out;
  a.target = (const Real*)target;
  a.grad = (Real*)grad_cells;
  a.loss_out = (Real*)loss_out;
  a.partials = (double*)scratch;
  a.counter = (unsigned*)(scratch + kCounterOffset);
  a.loss_w = loss_weight;
  a.inv_count = r->num_rays > 0 ? 1.0 / (4.0 * (double)r->num_rays) : std::nan("");
  if constexpr (std::is_same<Real, double>::value) {
    return launch_render_f64(a, g->mode, kTrain, stream);
  } else {
    if (g->dtype == PGB_BF16) return launch_render_bf16(a, g->mode, kTrain, stream);
    return launch_render_f32(a, g->mode, kTrain, stream);
  }
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" int pgb_render_train_noalloc(const pgb_grid* grid, const pgb_rays* rays,
                                        const void* target, double loss_weight, void* rgba_out,
                                        void* grad_cells, void* loss_out, pgb_stream_t stream) {
  // the same argument rules as pgb_render_train
  if (!grid || !grid->cells || !rays) return PGB_ERR_ARG;
  if (grid->dtype != PGB_F32 && grid->dtype != PGB_BF16 && grid->dtype != PGB_F64) return PGB_ERR_ARG;
  if (grid->mode != PGB_NEAREST && grid->mode != PGB_TRILINEAR) return PGB_ERR_ARG;
  if (grid->dims[0] <= 0 || grid->dims[1] <= 0 || grid->dims[2] <= 0) return PGB_ERR_ARG;
  if ((uint64_t)grid->dims[0] * grid->dims[1] * grid->dims[2] >= (1ull << 40)) return PGB_ERR_UNSUPPORTED;
  if (!aligned_to(grid->cells, grid->dtype == PGB_BF16 ? 8 : 16)) return PGB_ERR_ALIGN;
  if (rays->num_rays < 0 || rays->num_samples < 0) return PGB_ERR_ARG;
  if (rays->num_samples > kMaxSamples) return PGB_ERR_UNSUPPORTED;
  if (rays->log_transmittance) return PGB_ERR_UNSUPPORTED;  // product-scan form only
  // the scratch holds the loss partials of at most PGB_NOALLOC_MAX_RAYS rays per call
  if (rays->num_rays > PGB_NOALLOC_MAX_RAYS) return PGB_ERR_UNSUPPORTED;
  if (rays->cameras) {
    const pgb_cameras* c = rays->cameras;
    if (grid->dtype == PGB_F64) return PGB_ERR_UNSUPPORTED;
    if (!c->transforms || !c->images || c->num_cameras <= 0 || c->height <= 0 || c->width <= 0)
      return PGB_ERR_ARG;
    if (c->height != c->width) return PGB_ERR_UNSUPPORTED;
    if (!aligned_to(c->images, 16)) return PGB_ERR_ALIGN;
  } else if (rays->num_rays > 0 && (!rays->origins || !rays->dirs || !target)) {
    return PGB_ERR_ARG;
  }
  if (!grad_cells || !loss_out) return PGB_ERR_ARG;
  if (!aligned_to(grad_cells, 16)) return PGB_ERR_ALIGN;

  void* scratch = nullptr;
  int st = scratch_address(&scratch);
  if (st) return st;
  // the block counter must start at zero; every partial is written before it is read
  if (cudaMemsetAsync((unsigned char*)scratch + kCounterOffset, 0, sizeof(unsigned), stream) !=
      cudaSuccess)
    return PGB_ERR_LAUNCH;
  if (grid->dtype == PGB_F64)
    return launch_noalloc<double>(grid, rays, target, loss_weight, rgba_out, grad_cells, loss_out,
                                  (unsigned char*)scratch, stream);
  return launch_noalloc<float>(grid, rays, target, loss_weight, rgba_out, grad_cells, loss_out,
                               (unsigned char*)scratch, stream);
}
