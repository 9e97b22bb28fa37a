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

#include "pgb_host.h"
#include "render_args.cuh"

namespace pgb {
namespace {

// One ray per warp, so a call of at most PGB_NOALLOC_MAX_RAYS rays launches at most
// kNoAllocMaxBlocks blocks (of the smallest render block), each writing one loss partial.
constexpr int kNoAllocWarpsPerBlock = kRenderMinThreads / kWarp;
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

template <typename Real>
int launch_noalloc(const pgb_grid* g, const pgb_rays* r, const void* target, double loss_weight,
                   void* rgba_out, void* grad_cells, void* loss_out, unsigned char* scratch,
                   cudaStream_t stream) {
  // the same kernel arguments as pgb_render_train (render_args.cuh), with the loss
  // partials and the block counter in the library's scratch instead of a workspace
  RenderArgs<Real> a = render_args<Real>(g, r);
  const double samples = (double)r->num_rays * (double)r->num_samples;
  a.inv_samples = samples > 0 ? 1.0 / samples : std::nan("");
  a.rgba_out = (Real*)rgba_out;
  a.target = (const Real*)target;
  a.grad = (Real*)grad_cells;
  a.loss_out = (Real*)loss_out;
  a.partials = (double*)scratch;
  a.counter = (unsigned*)(scratch + kCounterOffset);
  a.loss_w = loss_weight;
  a.inv_count = r->num_rays > 0 ? 1.0 / (4.0 * (double)r->num_rays) : std::nan("");
  return dispatch_render<Real>(g, r, a, kTrain, stream);
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" int pgb_render_train_noalloc(const pgb_grid* grid, const pgb_rays* rays,
                                        const void* target, double loss_weight, void* rgba_out,
                                        void* grad_cells, void* loss_out, pgb_stream_t stream) {
  // the same argument rules as pgb_render_train
  int st = check_grid(grid);
  if (st) return st;
  if ((st = check_rays(grid, rays, true))) return st;
  // the scratch holds the loss partials of at most PGB_NOALLOC_MAX_RAYS rays per call
  if (rays->num_rays > PGB_NOALLOC_MAX_RAYS) return PGB_ERR_UNSUPPORTED;
  if (!grad_cells || !loss_out) return PGB_ERR_ARG;
  if (!rays->cameras && rays->num_rays > 0 && !target) return PGB_ERR_ARG;
  if (!aligned(grad_cells, 16)) return PGB_ERR_ALIGN;

  void* scratch = nullptr;
  if ((st = scratch_address(&scratch))) return st;
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
