// Compile-time dispatch of the fused render kernel over lookup mode, phase and slots per
// lane. Included once per storage type (render_f32.cu, render_bf16.cu, render_f64.cu) and
// per storage type for the log-sum transmittance form (render_logt_*.cu) so the instantiations compile
// in parallel.
#pragma once

#include <algorithm>

#include "pgb_host.h"
#include "render.cuh"

namespace pgb {

template <typename Real, typename Store, int MODE, int K, int PHASE, bool LOGT>
int launch_render_k(const RenderArgs<Real>& a, cudaStream_t s) {
  constexpr int kThreads = render_threads<MODE, K>();
  constexpr int kWarpsPerBlock = kThreads / kWarp;
  constexpr int kSmem = render_smem_bytes<Real, K, LOGT>(kWarpsPerBlock);
  // the dynamic shared-memory opt-in (dynamic + static may pass 48 KiB) is per device:
  // set it on first use of each device
  static int configured[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    if (cudaFuncSetAttribute(render_kernel<Real, Store, MODE, K, PHASE, LOGT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem) != cudaSuccess)
      return PGB_ERR_LAUNCH;
    configured[dev] = 1;
  }
  int64_t blocks = (a.R + kWarpsPerBlock - 1) / kWarpsPerBlock;
  blocks = std::min<int64_t>(blocks, PHASE == kTrain ? kMaxTrainWarps / kWarpsPerBlock
                                                     : (int64_t)1 << 20);
  if (blocks < 1) blocks = 1;
  render_kernel<Real, Store, MODE, K, PHASE, LOGT><<<(unsigned)blocks, kThreads, kSmem, s>>>(a);
  return after_launch();
}

template <typename Real, typename Store, int MODE, int PHASE, bool LOGT>
int launch_render_mp(const RenderArgs<Real>& a, cudaStream_t s) {
  const bool early_stop = a.g.clip && !(PHASE == kTrain && a.beta_w != 0.0);
  switch (pick_slots(a.S, a.chunk_samples, early_stop, MODE)) {
    case 1: return launch_render_k<Real, Store, MODE, 1, PHASE, LOGT>(a, s);
    case 2: return launch_render_k<Real, Store, MODE, 2, PHASE, LOGT>(a, s);
    case 4: return launch_render_k<Real, Store, MODE, 4, PHASE, LOGT>(a, s);
    case 8: return launch_render_k<Real, Store, MODE, 8, PHASE, LOGT>(a, s);
    case 16: return launch_render_k<Real, Store, MODE, 16, PHASE, LOGT>(a, s);
    default: return PGB_ERR_UNSUPPORTED;
  }
}

template <typename Real, typename Store, bool LOGT = false>
int launch_render_t(const RenderArgs<Real>& a, int mode, int phase, cudaStream_t s) {
  if (mode == PGB_NEAREST) {
    if (phase == kForward) return launch_render_mp<Real, Store, PGB_NEAREST, kForward, LOGT>(a, s);
    if (phase == kBackward) return launch_render_mp<Real, Store, PGB_NEAREST, kBackward, LOGT>(a, s);
    if (phase == kTrain) return launch_render_mp<Real, Store, PGB_NEAREST, kTrain, LOGT>(a, s);
  } else if (mode == PGB_TRILINEAR) {
    if (phase == kForward) return launch_render_mp<Real, Store, PGB_TRILINEAR, kForward, LOGT>(a, s);
    if (phase == kBackward) return launch_render_mp<Real, Store, PGB_TRILINEAR, kBackward, LOGT>(a, s);
    if (phase == kTrain) return launch_render_mp<Real, Store, PGB_TRILINEAR, kTrain, LOGT>(a, s);
  }
  return PGB_ERR_ARG;
}

}  // namespace pgb
